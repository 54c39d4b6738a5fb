"""Failure paths on the GPU, without a fault: bounded loops and waits that
run out set error bits which the host reads, and the device stays usable.

  * Ray-march step bound: a sampling rate so high that a ray would need
    millions of steps stops at the bound and sets bit 16 of the frame's
    errorFlags (reported through the status callback), in the volume-only
    marcher and in the per-pixel raycast kernel; the next frame at a sane
    rate is clean and matches the oracle.
  * tcgen05 waits: vsrDenoiserTestWaitTimeout makes the MMA thread of every
    CTA of the next tcgen05 convolution wait on a barrier that nothing
    completes; the one-second wait runs out, the launch ends early, the
    error word reads 1 (vsrDenoiseFrame returns VSR_ERROR_TIMEOUT), and the
    following pass matches the CPU restatement with a clean error word. Both
    tcgen05 kernels (warp-specialised TMA, one tile per CTA).
"""
import numpy as np
import pytest

import denoise_oracle as D

pytestmark = pytest.mark.gpu

ERR_MARCH_LIMIT = 16
VSR_ERROR_TIMEOUT = 7


def _release(device, h):
    for o in (h["frame"], h["renderer"], h["camera"], h["world"], *h["keep"]):
        device.release(o)


@pytest.mark.parametrize("surfaces", [False, True])
def test_march_step_limit_sets_error_flag(pkg, device, oracle, surfaces):
    sc = pkg.scenes.config0(res=24, n=32)
    if surfaces:  # a world with surfaces takes the per-pixel raycast kernel
        sc["surfaces"] = [{"vertices": np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32),
                           "indices": np.array([[0, 1, 2]], np.uint32),
                           "material": {"type": "matte", "color": [0.5, 0.5, 0.5]}}]
    sc["renderer"]["volumeSamplingRate"] = 2.0e7  # dt = 5e-8 voxel: ~6e8 steps per ray
    h = pkg.scenes.build(device, sc, channels=("color", "depth"))
    n0 = len(device.messages)
    assert device.render(h["frame"]) == 0
    assert device.wait(h["frame"])
    flags = device.get_uint(h["frame"], "errorFlags")
    assert flags & ERR_MARCH_LIMIT, flags
    assert any("error flags" in m[2] for m in device.messages[n0:])
    # the same frame at the configured rate: clean, and equal to the oracle
    device.set(h["renderer"], "volumeSamplingRate", 2.0)
    device.commit(h["renderer"])
    assert device.render(h["frame"]) == 0
    assert device.wait(h["frame"])
    assert device.get_uint(h["frame"], "errorFlags") == 0
    color = device.map(h["frame"], "channel.color")
    _release(device, h)
    sc["renderer"]["volumeSamplingRate"] = 2.0
    S = oracle.Scene(sc)
    F = oracle.Frame(24, 24)
    oracle.render(S, F)
    assert float((np.abs(color - F.color).max(axis=-1) <= 2e-3).mean()) >= 0.999


def _forward_case(seed=3):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, 1, (1, 16, 256, 16)).astype(np.float32)
    x[..., 10:] = 0.0
    x = D.bf16(x)
    params = D.init_params(5)
    params[np.arange(len(params)) % 11 == 0] += 0.02
    return x, params


@pytest.mark.parametrize("path", [1, 3])
def test_denoiser_wait_timeout_is_reported_and_recovered(pkg, device, path):
    import torch
    x, params = _forward_case()
    dn = pkg.vsr.Denoiser(device, seed=1)
    try:
        dn.set_tensor_path(path)
        dn.set_params(params)
        assert dn.errors() == 0
        xd = torch.from_numpy(x).to(torch.bfloat16).cuda().contiguous()
        out = torch.zeros((1, 16, 256, 16), dtype=torch.float32, device="cuda")
        dn.test_wait_timeout()
        dn.forward(xd.data_ptr(), 1, 16, 256, out.data_ptr())
        torch.cuda.synchronize()
        assert dn.errors() == 1
        assert dn.errors() == 0  # reading cleared it
        # the next pass runs normally
        out.zero_()
        dn.forward(xd.data_ptr(), 1, 16, 256, out.data_ptr())
        torch.cuda.synchronize()
        assert dn.errors() == 0
        ref = D.forward(params, x)["out"][..., :3]
        err = float(np.abs(out.cpu().numpy()[..., :3] - ref).max())
        assert err <= 2e-2 * float(np.abs(ref).max()) + 1e-3, err
    finally:
        dn.close()


def test_denoise_frame_returns_timeout(pkg, device):
    """vsrDenoiseFrame (synchronous with a retry count) turns the error word
    into VSR_ERROR_TIMEOUT and a status message; the next call succeeds."""
    import torch
    sc = pkg.scenes.config1(res=128, spp=4, num_spheres=8, nu=16, nv=8)
    h = pkg.scenes.build(device, sc)
    assert device.render(h["frame"]) == 0
    assert device.wait(h["frame"])
    dn = pkg.vsr.Denoiser(device, seed=1)
    try:
        out = torch.zeros((128 * 128, 4), dtype=torch.float32, device="cuda")
        dn.test_wait_timeout()
        n0 = len(device.messages)
        with pytest.raises(RuntimeError, match=f"\\({VSR_ERROR_TIMEOUT}\\)"):
            dn.denoise_frame(h["frame"], out.data_ptr())
        assert any("wait ran out" in m[2] for m in device.messages[n0:])
        assert dn.errors() == 1
        dn.denoise_frame(h["frame"], out.data_ptr())
        assert dn.errors() == 0
        assert torch.isfinite(out).all()
    finally:
        dn.close()
        _release(device, h)
