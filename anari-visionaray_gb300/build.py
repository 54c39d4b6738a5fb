"""Build the renderer core library (libvsr.so) in-tree for sm_103a, and
libvsr_probe.so (single device functions behind test entry points).

Compiles the CUDA translation units with nvcc and the host runtime with g++
in parallel, then links one shared library next to this file. Objects go to
_build/ (git-ignored). Re-running only recompiles what changed.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvsr.so")
# probe entry points of single device functions, loaded by tests only
PROBE_LIB = os.path.join(HERE, "libvsr_probe.so")
PROBE_SOURCES = ["probe.cu"]
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE, *ARCH]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-Wall", "-I" + INCLUDE]

CU_SOURCES = ["k_render.cu", "k_wavefront.cu", "k_bvh.cu", "k_bvh_ploc.cu", "k_bvh4.cu", "k_bvh_leaves.cu", "k_bvh_noalloc.cu", "k_volume.cu", "k_volume_march.cu", "k_batch.cu", "k_denoise.cu", "k_denoise_tc.cu", "k_denoise_ws.cu", "k_denoise_wg.cu"]
CPP_SOURCES = ["runtime.cpp", "denoiser.cpp"]
HEADERS = ["vsr_device.h", "render_common.cuh", "render_pixel.cuh", "kernels.h", "bvh_kernels.cuh", "denoiser.h"]


def _cuda_home():
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _newest_dep_mtime():
    paths = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "vsr.h")]
    return max(os.path.getmtime(p) for p in paths)


def _stale(src, obj, dep_mtime):
    if not os.path.exists(obj):
        return True
    return os.path.getmtime(obj) < max(os.path.getmtime(src), dep_mtime)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build(verbose=False):
    """Compile and link libvsr.so; returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    dep = _newest_dep_mtime()
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(OBJ, s + ".o")
        objs.append(obj)
        if _stale(src, obj, dep):
            jobs.append([nvcc, *NVCC_FLAGS, "-c", src, "-o", obj])
    probe_objs = []
    for s in PROBE_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(OBJ, s + ".o")
        probe_objs.append(obj)
        if _stale(src, obj, dep):
            jobs.append([nvcc, *NVCC_FLAGS, "-c", src, "-o", obj])
    for s in CPP_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(OBJ, s + ".o")
        objs.append(obj)
        if _stale(src, obj, dep):
            jobs.append(["g++", *CXX_FLAGS, "-I" + os.path.join(cuda, "include"), "-c", src, "-o", obj])
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for f in [ex.submit(_run, j, verbose) for j in jobs]:
            f.result()
    if jobs or not os.path.exists(LIB):
        _run([nvcc, "-shared", *ARCH, "-o", LIB, *objs], verbose)
    if jobs or not os.path.exists(PROBE_LIB):
        _run([nvcc, "-shared", *ARCH, "-o", PROBE_LIB, *probe_objs], verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
