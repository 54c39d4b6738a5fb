"""Batched rendering (vsrRenderFrames) against per-frame rendering.

Frames of different scenes, renderers (path tracer and raycast, with and
without surfaces), sizes and sample counts are rendered twice: each on its
own through vsrRenderFrame, and all together through vsrRenderFrames. Both
run the same per-pixel bodies with the same random streams; they are
compiled into different kernels, where the compiler may fuse a different
product of an `a*b + c*d` into a multiply-add, so single bits of a result
can differ (a volume march compounds them over hundreds of samples), and a
path-tracer sample whose random decision sits on such a bit can take
another path. The test therefore asks for equality up to that: every
channel within 1e-3 on 99.5 % of pixels and no NaN, over successive
accumulated frames, while the batch autotuner steps through its
configurations and after it has settled.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CHANNELS = ("color", "depth", "normal", "albedo")


def small_batch(pkg):
    scenes = pkg.scenes.config3(num_scenes=6, sizes=(40, 64, 96), side=(24, 48),
                                tris=(4000, 20000), spp=(1, 4))
    # cover every kind: raycast volume-only, raycast with surfaces, path
    # tracing with and without surfaces
    with_s = [s for s in scenes if s["surfaces"]]
    without = [s for s in scenes if not s["surfaces"]]
    assert with_s and len(without) >= 2

    def as_kind(s, kind):
        s = dict(s)
        r = dict(s["renderer"], type=kind)
        if kind == "pathtrace":
            r["maxBounce"] = 3
        s["renderer"] = r
        return s

    return [as_kind(without[0], "raycast"), as_kind(with_s[0], "raycast"),
            as_kind(with_s[0], "pathtrace"), as_kind(without[1], "pathtrace")] + \
        [as_kind(s, s["renderer"]["type"]) for s in scenes[:2]]


def same_bits(x, y, what):
    """Within 1e-3 on >= 99.5 % of pixels, no NaN; prints the bit-identical share."""
    assert x.shape == y.shape, what
    px = x.reshape(x.shape[0], x.shape[1], -1)
    py = y.reshape(px.shape)
    exact = np.all(px.view(np.uint32) == py.view(np.uint32), axis=-1)
    close = np.all(np.abs(px.astype(np.float64) - py.astype(np.float64)) <= 1e-3, axis=-1)
    big = np.abs(px) > 1e30  # the 1e31 "no hit" depth
    close |= np.all(big == (np.abs(py) > 1e30), axis=-1) & np.all(big, axis=-1)
    print(f"{what}: exact {exact.mean():.4f} close {close.mean():.4f}")
    assert not np.isnan(py).any(), what
    assert close.mean() >= 0.995, what


def release(dev, h):
    for o in (h["frame"], h["renderer"], h["camera"], h["world"], *h["keep"]):
        dev.release(o)


def test_batch_matches_single_frames(pkg, device):
    dev = device
    scenes = small_batch(pkg)
    single = [pkg.scenes.build(dev, s, channels=CHANNELS) for s in scenes]
    batch = [pkg.scenes.build(dev, s, channels=CHANNELS) for s in scenes]
    frames = [h["frame"] for h in batch]
    try:
        for it in range(11):  # the tuner tries 8 configurations, then settles
            for h in single:
                assert dev.render(h["frame"]) == 0
            assert dev.render_batch(frames) == 0
            for h in single + batch:
                dev.wait(h["frame"])
            for k, (a, b) in enumerate(zip(single, batch)):
                assert dev.get_uint(b["frame"], "errorFlags") == 0
                for ch in CHANNELS:
                    x, y = dev.map(a["frame"], "channel." + ch), dev.map(b["frame"], "channel." + ch)
                    same_bits(x, y, f"frame {k} ({scenes[k]['renderer']['type']}) {ch} batch {it}")
            assert dev.get_int(frames[0], "numSamples") == it + 1
        assert dev.get_int(frames[0], "batch.tuned") == 1
        assert 32 % dev.get_int(frames[0], "batch.tileWidth") == 0
    finally:
        for h in single + batch:
            release(dev, h)


def test_batch_gradient_shading(pkg, device):
    """Raycast and path-traced frames with gradient shading batched beside an
    unshaded raycast frame (the shaded frames take their own kernel variants):
    the same images as rendered one at a time."""
    dev = device
    base = small_batch(pkg)

    def shaded(s):
        return dict(s, renderer=dict(s["renderer"], gradientShading=True))

    # and a frame of each renderer over sphere geometry (full variants too)
    rng = np.random.default_rng(5)
    balls = {"geometry": "sphere", "vertices": rng.uniform(-10.0, 10.0, (24, 3)).astype(np.float32),
             "radii": rng.uniform(1.0, 4.0, 24).astype(np.float32),
             "material": {"type": "matte", "color": [0.7, 0.6, 0.5]}}
    with_balls = [dict(base[k], surfaces=list(base[k]["surfaces"]) + [balls]) for k in (0, 3)]
    scenes = [shaded(base[0]), shaded(base[1]), shaded(base[3]), base[0]] + with_balls
    single = [pkg.scenes.build(dev, s, channels=CHANNELS) for s in scenes]
    batch = [pkg.scenes.build(dev, s, channels=CHANNELS) for s in scenes]
    frames = [h["frame"] for h in batch]
    try:
        for it in range(3):
            for h in single:
                assert dev.render(h["frame"]) == 0
            assert dev.render_batch(frames) == 0
            for h in single + batch:
                dev.wait(h["frame"])
            for k, (a, b) in enumerate(zip(single, batch)):
                assert dev.get_uint(b["frame"], "errorFlags") == 0
                for ch in CHANNELS:
                    x, y = dev.map(a["frame"], "channel." + ch), dev.map(b["frame"], "channel." + ch)
                    same_bits(x, y, f"shaded frame {k} {ch} batch {it}")
        # the shading changed the raycast image
        a = dev.map(batch[0]["frame"], "channel.color")
        b = dev.map(batch[3]["frame"], "channel.color")
        assert np.abs(a[..., :3] - b[..., :3]).max() > 1e-2
    finally:
        for h in single + batch:
            release(dev, h)


def test_batch_commit_resets_accumulation(pkg, device):
    """A commit to one frame's camera restarts that frame's accumulation in
    the batch exactly as vsrRenderFrame does."""
    dev = device
    scenes = small_batch(pkg)[2:4]
    single = [pkg.scenes.build(dev, s, channels=("color",)) for s in scenes]
    batch = [pkg.scenes.build(dev, s, channels=("color",)) for s in scenes]
    try:
        for it in range(3):
            if it == 2:
                for h in (single[0], batch[0]):
                    dev.set(h["camera"], "fovy", 0.5)
                    dev.commit(h["camera"])
            for h in single:
                dev.render(h["frame"])
            dev.render_batch([h["frame"] for h in batch])
            for h in single + batch:
                dev.wait(h["frame"])
        assert dev.get_int(batch[0]["frame"], "numSamples") == 1
        assert dev.get_int(batch[1]["frame"], "numSamples") == 3
        for k, (a, b) in enumerate(zip(single, batch)):
            same_bits(dev.map(a["frame"], "channel.color"), dev.map(b["frame"], "channel.color"),
                      f"frame {k} after reset")
    finally:
        for h in single + batch:
            release(dev, h)
