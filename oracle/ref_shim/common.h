// Test infrastructure: stands in for the reference's top-level common.h
// (which needs the ANARI SDK and Visionaray) when the reference's
// frame/common.h is compiled; it provides only the shim math types.
#pragma once
#include "vsnray_shim.h"
