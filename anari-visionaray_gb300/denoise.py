"""Training data, training and evaluation of the learned denoiser.

Everything that computes runs through the renderer core's C ABI: the path
tracer renders the low/high-sample pairs, vsrDenoiserFrameInput builds the
network inputs, vsrDenoiserTrainStep runs forward, backward and Adam, and
vsrDenoiseFrame denoises and applies the variance gate. torch only holds
device buffers (and cuts training crops out of them).

Scenes come from the config-1/2 generators with per-scene seeds: a random
UV-sphere set (32 x 16 segments), a value-noise volume in half of them,
a random camera orbit and light direction. Inputs are the accumulated
images after a few samples per pixel (4 to 32); references are
accumulated high-sample renders of the same view.
"""
import math
import time

import numpy as np

from . import scenes, vsr

CHANNELS = ("color", "depth", "normal", "albedo")


def training_scene(seed, res=256, spp=4, max_bounce=5):
    """One random scene in the style of configs 1 and 2, seeded by `seed`."""
    rng = np.random.default_rng(seed)
    num = int(rng.integers(12, 64))
    surfaces = scenes.sphere_set(rng, num, nu=32, nv=16)
    volumes = []
    if rng.uniform() < 0.5:
        n = 64
        data = scenes.value_noise(n, rng, octaves=4)
        color, opacity = scenes.smoke_tf(alpha_max=float(rng.uniform(0.2, 0.6)))
        spacing = 24.0 / (n - 1)
        volumes.append({"data": data, "origin": [-12.0] * 3, "spacing": [spacing] * 3,
                        "color": color, "opacity": opacity, "valueRange": [0.0, 1.0],
                        "unitDistance": float(1.0 / rng.uniform(5.0, 40.0)),
                        "majorantBrickSize": 16})
    theta = rng.uniform(0, 2 * math.pi)
    dist = rng.uniform(26.0, 40.0)
    height = rng.uniform(2.0, 16.0)
    eye = [dist * math.sin(theta), height, dist * math.cos(theta)]
    ld = np.array([rng.uniform(-0.6, 0.6), -1.0, rng.uniform(-0.6, 0.6)])
    ld /= np.linalg.norm(ld)
    return {
        "surfaces": surfaces, "volumes": volumes,
        "lights": [{"direction": [float(x) for x in ld], "color": [1.0, 1.0, 1.0],
                    "irradiance": float(rng.uniform(2.0, 4.0))}],
        "camera": scenes._look_at_camera([0.0, -1.0, 0.0], eye, 45.0, 1.0),
        "renderer": {"type": "pathtrace", "pixelSamples": spp, "maxBounce": max_bounce,
                     "ambientRadiance": float(rng.uniform(0.1, 0.3)), "background": [0, 0, 0, 1]},
        "frame": {"size": (res, res)},
    }


def _second_frame(dev, h, spp):
    """A colour-only frame of the same world and camera with its own renderer."""
    rend = dev.renderer("pathtrace")
    scenes.apply_renderer(dev, rend, dict(h["scene"]["renderer"], pixelSamples=spp))
    frame = dev.frame()
    W, H = h["scene"]["frame"]["size"]
    dev.set(frame, "size", (W, H), vsr.UINT32_VEC2)
    dev.set(frame, "channel.color", vsr.FLOAT32_VEC4, vsr.DATA_TYPE)
    dev.set(frame, "world", h["world"])
    dev.set(frame, "camera", h["camera"])
    dev.set(frame, "renderer", rend)
    dev.commit(frame)
    return rend, frame


def render_reference(dev, h, spp_total, per_frame=256):
    """The accumulated mean of spp_total samples per pixel, (H, W, 4) float32."""
    rend, frame = _second_frame(dev, h, min(per_frame, spp_total))
    for _ in range(max(1, spp_total // per_frame)):
        dev.render(frame)
    dev.wait(frame)
    ref = dev.map(frame, "channel.color")
    dev.release(frame)
    dev.release(rend)
    return ref


def build(dev, scene, variance=True):
    """The scene's objects with colour, depth, normal and albedo channels
    (and the variance channel)."""
    h = scenes.build(dev, scene, channels=CHANNELS)
    if variance:
        dev.set(h["frame"], "channel.variance", vsr.FLOAT32, vsr.DATA_TYPE)
        dev.commit(h["frame"])
    h["scene"] = scene
    return h


def release(dev, h):
    for o in (h["frame"], h["renderer"], h["camera"], h["world"], *h["keep"]):
        dev.release(o)


def make_dataset(dev, seeds, res=256, ref_spp=1024, input_spp=(4,)):
    """Network inputs (N * L, res, res, 16) bf16 and their reference colours
    (N * L, res, res, 4) fp32 on the GPU, rendered by the path tracer: for
    each scene, the inputs after each of the L sample counts input_spp
    (ascending, multiples of 4) of one accumulating frame, all with the
    same reference."""
    import torch

    levels = sorted(input_spp)
    n = len(seeds) * len(levels)
    x = torch.zeros((n, res, res, vsr.Denoiser.IN_C), dtype=torch.bfloat16, device="cuda")
    t = torch.zeros((n, res, res, 4), dtype=torch.float32, device="cuda")
    i = 0
    for seed in seeds:
        h = build(dev, training_scene(seed, res, 4), variance=True)
        ref = torch.from_numpy(render_reference(dev, h, ref_spp)).cuda()
        done = 0
        for s in levels:
            while done < s:
                dev.render(h["frame"])
                done += 4
            dev.wait(h["frame"])
            torch.cuda.synchronize()
            dev.denoise_input(h["frame"], x[i].data_ptr())
            dev.wait(h["frame"])
            t[i] = ref
            i += 1
        release(dev, h)
    torch.cuda.synchronize()
    return x, t


def train(dn, x, t, steps, batch=16, crop=128, lr=1e-3, seed=0, log_every=0, warmup=None):
    """Adam on random crops, the learning rate rising linearly over the first
    `warmup` steps (default 5 %) and then decaying on a cosine; returns the
    logged (step, loss) pairs and the wall time. Without the warm-up, Adam's
    first steps (each weight moved by the full rate) can switch every ReLU
    off, which leaves the residual network at the identity."""
    import torch

    g = torch.Generator(device="cpu")
    g.manual_seed(seed)
    n, H, W, _ = x.shape
    # every step's crops (image, row, column), drawn in the order of one
    # step after another, moved to the device once
    picks = []
    for _ in range(steps):
        idx = torch.randint(0, n, (batch,), generator=g)
        oy = torch.randint(0, (H - crop) // 8 + 1, (batch,), generator=g) * 8
        ox = torch.randint(0, (W - crop) // 8 + 1, (batch,), generator=g) * 8
        picks.append(torch.stack([idx, oy, ox]))
    picks = torch.stack(picks).to(x.device)  # (steps, 3, batch)
    ar = torch.arange(crop, device=x.device)
    losses = []
    # the crops are gathered on the device's own stream, so each step's
    # kernels follow its gather without a host synchronisation; the loss is
    # read back (which waits for the step) only where it is logged
    stream = torch.cuda.ExternalStream(dn.dev.lib.vsrDeviceStream(dn.dev.handle))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for s in range(steps):
            idx, oy, ox = picks[s]
            rows = (oy[:, None] + ar[None, :])[:, :, None]
            cols = (ox[:, None] + ar[None, :])[:, None, :]
            xb = x[idx[:, None, None], rows, cols].contiguous()
            tb = t[idx[:, None, None], rows, cols].contiguous()
            ramp = min(1.0, (s + 1) / max(1, warmup if warmup is not None else steps // 20))
            rate = lr * ramp * 0.5 * (1.0 + math.cos(math.pi * s / steps))
            want = (bool(log_every) and s % log_every == 0) or s == steps - 1
            loss = dn.train_step(xb.data_ptr(), tb.data_ptr(), 4, batch, crop, crop, rate,
                                 want_loss=want)
            if want and log_every:
                losses.append((s, loss))
    return losses, time.perf_counter() - t0


def sq_errors(a, b):
    """Sums of squared errors of the colour channels: linear, and after the
    Reinhard tone map c / (1 + c), which bounds the rare very bright
    samples ("fireflies") that otherwise dominate a linear RMSE."""
    x, y = a[..., :3].astype(np.float64), b[..., :3].astype(np.float64)
    d = x - y
    tm = np.clip(x, 0, None) / (1 + np.clip(x, 0, None)) - np.clip(y, 0, None) / (1 + np.clip(y, 0, None))
    return float(np.sum(d * d)), float(np.sum(tm * tm))


def evaluate(dev, dn, seeds, res=256, ref_spp=4096, spp_levels=(4, 8, 16, 32, 64, 128, 256),
             denoise_levels=(4, 8, 16), k=3.0, floor=0.01):
    """Pooled errors against ref_spp references of plain path tracing at
    spp_levels, of the denoised image at denoise_levels, and of the
    variance-gated image, with the share of pixels the gate sends back for
    more samples. Returns {"plain" | "denoised" | "gated": {"rmse": {spp:
    linear RMSE}, "rmse_tm": {spp: tone-mapped RMSE}, "psnr_tm": {spp: dB}},
    "retry": {spp: share}}."""
    import torch

    kinds = ("plain", "denoised", "gated")
    sums = {kd: {} for kd in kinds}
    retry = {s: 0 for s in denoise_levels}
    npx = 0
    out = torch.zeros((res * res, 4), dtype=torch.float32, device="cuda")

    def add(kind, s, img, ref):
        lin, tm = sq_errors(img, ref)
        a = sums[kind].setdefault(s, [0.0, 0.0])
        a[0] += lin
        a[1] += tm

    for seed in seeds:
        h = build(dev, training_scene(seed, res, 4), variance=True)
        ref = render_reference(dev, h, ref_spp)
        done = 0
        for s in sorted(set(spp_levels) | set(denoise_levels)):
            while done < s:
                dev.render(h["frame"])
                done += 4
            dev.wait(h["frame"])
            if s in spp_levels:
                add("plain", s, dev.map(h["frame"], "channel.color"), ref)
            if s in denoise_levels:
                dn.denoise_frame(h["frame"], out.data_ptr(), k=1e30, floor=0.0)
                add("denoised", s, out.cpu().numpy().reshape(res, res, 4), ref)
                retry[s] += dn.denoise_frame(h["frame"], out.data_ptr(), k=k, floor=floor)
                add("gated", s, out.cpu().numpy().reshape(res, res, 4), ref)
        npx += res * res
        release(dev, h)
    n = 3.0 * npx
    res_ = {}
    for kd in kinds:
        rm = {s: math.sqrt(v[0] / n) for s, v in sorted(sums[kd].items())}
        rt = {s: math.sqrt(v[1] / n) for s, v in sorted(sums[kd].items())}
        res_[kd] = {"rmse": rm, "rmse_tm": rt,
                    "psnr_tm": {s: (20 * math.log10(1.0 / v) if v > 0 else float("inf"))
                                for s, v in rt.items()}}
    res_["retry"] = {s: v / npx for s, v in retry.items()}
    return res_


def time_to_rmse(plain, dn, pt_s_per_spp, dn_s, target_spp=256):
    """Time for plain path tracing to reach its target_spp error, and for
    denoised path tracing (the fewest input samples whose denoised error is
    at most that) to reach it, from per-sample render time and denoiser
    time; plain and dn map spp to an error (e.g. tone-mapped RMSE). Returns
    (goal error, plain seconds, input spp or None, denoised seconds or
    None)."""
    goal = plain[target_spp]
    t_plain = target_spp * pt_s_per_spp
    ok = [s for s in sorted(dn) if dn[s] <= goal]
    if not ok:
        return goal, t_plain, None, None
    s = ok[0]
    return goal, t_plain, s, s * pt_s_per_spp + dn_s


def plain_spp_for(plain, err):
    """Samples per pixel plain path tracing needs for the error `err`, from
    its measured error curve (spp -> error): log-log interpolation between
    the measured levels, beyond the last one the Monte-Carlo rate error ~
    1/sqrt(spp) from the last level."""
    pts = sorted(plain.items())
    if err >= pts[0][1]:
        return float(pts[0][0])
    for (s0, e0), (s1, e1) in zip(pts, pts[1:]):
        if e1 <= err <= e0:
            if e0 == e1:
                return float(s0)
            f = math.log(e0 / err) / math.log(e0 / e1)
            return float(math.exp(math.log(s0) + f * math.log(s1 / s0)))
    s_last, e_last = pts[-1]
    return float(s_last * (e_last / err) ** 2)


def at_input_spp(plain, dn, pt_s_per_spp, dn_s, spp=4):
    """What denoising `spp` input samples buys: its error, the plain sample
    count with the same error, and the time ratio of the two at that error
    (plain spp_equal x per-sample time vs spp x per-sample time + the
    denoiser pass)."""
    e = dn[spp]
    s_eq = plain_spp_for(plain, e)
    t_plain = s_eq * pt_s_per_spp
    t_dn = spp * pt_s_per_spp + dn_s
    return {"input_spp": spp, "denoised_rmse_tm": e, "plain_spp_same_rmse": s_eq,
            "plain_s_1080p": t_plain, "denoised_s_1080p": t_dn,
            "speedup_at_that_rmse": t_plain / t_dn}


def evaluate_gated_loop(dev, dn, seeds, res=256, ref_spp=4096, input_spp=4, rounds=4,
                        frames_per_round=4, k=3.0, floor=0.01):
    """The variance gate as a loop: after input_spp samples per pixel (one
    frame of 4 spp per 4 samples), denoise and gate; the pixels the gate
    rejects get frames_per_round more frames (4 spp each) through the
    frame's sample mask (vsrFrameSampleMask), then the frame is denoised and
    gated again, up to `rounds` times. Per round r (0 = after the input
    samples only), pooled over the scenes: the tone-mapped RMSE of the gated
    image against ref_spp references, the share of pixels the gate sent
    back, and the samples per pixel spent so far (all pixels' input samples
    plus the rejected pixels' extra ones, divided by the pixel count)."""
    import torch

    npx = res * res
    sq = {}
    spent = {}
    retried = {}
    mask = torch.zeros(npx, dtype=torch.uint8, device="cuda")
    out = torch.zeros((npx, 4), dtype=torch.float32, device="cuda")
    for seed in seeds:
        h = build(dev, training_scene(seed, res, 4), variance=True)
        ref = render_reference(dev, h, ref_spp)
        for _ in range(max(1, input_spp // 4)):
            dev.render(h["frame"])
        dev.wait(h["frame"])
        px_spp = float(npx * input_spp)
        for r in range(rounds + 1):
            nret = dn.denoise_frame(h["frame"], out.data_ptr(), k=k, floor=floor,
                                    retry_ptr=mask.data_ptr())
            img = out.cpu().numpy().reshape(res, res, 4)
            sq[r] = sq.get(r, 0.0) + sq_errors(img, ref)[1]
            spent[r] = spent.get(r, 0.0) + px_spp
            retried[r] = retried.get(r, 0) + nret
            if r == rounds:
                break
            dev.sample_mask(h["frame"], mask.data_ptr())
            for _ in range(frames_per_round):
                dev.render(h["frame"])
            dev.wait(h["frame"])
            px_spp += float(nret) * 4 * frames_per_round
        dev.sample_mask(h["frame"], None)
        release(dev, h)
    n = len(seeds)
    return [{"round": r, "rmse_tm": math.sqrt(sq[r] / (3.0 * npx * n)),
             "retry_share": retried[r] / (npx * n), "spp_per_pixel": spent[r] / (npx * n)}
            for r in sorted(sq)]


def gated_loop_times(loop, pt_s_per_spp, dn_s, masked_s_per_px_spp, px_1080p=1920 * 1080,
                     frames_per_round=4):
    """Seconds at 1920x1080 to reach each round of evaluate_gated_loop: the
    input samples over every pixel, the rejected pixels' extra samples at
    the measured per-pixel-sample cost of masked frames, and one denoiser
    pass per round."""
    out = []
    for e in loop:
        r = e["round"]
        t = loop[0]["spp_per_pixel"] * pt_s_per_spp + (r + 1) * dn_s
        for q in loop[:r]:
            t += q["retry_share"] * px_1080p * 4 * frames_per_round * masked_s_per_px_spp
        out.append(dict(e, s_1080p=t))
    return out
