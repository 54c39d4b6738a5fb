"""GPU parity: the CUDA renderer core (through the C ABI) against the CPU
oracle on the same seeded scenes.

Tolerances (from the project's parity bar):
  raycast    : per-channel |delta| <= 2e-3 on >= 99.9 % of pixels; depth within
               1e-4 relative on surface-hit pixels (volume-only frames write 1e31).
  pathtracer : the GPU mean image lies inside the oracle's per-pixel 3 sigma band
               (sigma from per-sample variance of both estimates) on >= 98.5 % of
               pixels for independent random streams; with the same stream the
               GPU reproduces the oracle sample for sample (>= 97 % of pixels
               within 1e-3), since both follow the reference's per-pixel LCG.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RAYCAST_TOL = 2e-3


def render_gpu(pkg, dev, scene, frames=1, accum_offset=0):
    h = pkg.scenes.build(dev, scene)
    for _ in range(frames):
        assert dev.render(h["frame"]) == 0
        assert dev.wait(h["frame"])
    out = {c: dev.map(h["frame"], "channel." + c) for c in ("color", "depth", "normal", "albedo")}
    out["errorFlags"] = dev.get_uint(h["frame"], "errorFlags")
    for o in (h["frame"], h["renderer"], h["camera"], h["world"]):
        dev.release(o)
    for o in h["keep"]:
        dev.release(o)
    return out


def render_oracle(oracle, scene, frames=1, accum_start=0, stats=False, grid=None, tile=None):
    kw = {} if grid is None else {"grid_method": grid}
    S = oracle.Scene(scene, **kw)
    W, H = scene["frame"]["size"]
    F = oracle.Frame(W, H, stats=stats)
    F.f.accumID = accum_start
    for _ in range(frames):
        oracle.render(S, F, tile=tile)
    return S, F


def raycast_ok(gpu, F, tol=RAYCAST_TOL, frac=0.999):
    d = np.abs(gpu["color"] - F.color).max(axis=-1)
    ok = float((d <= tol).mean())
    return ok >= frac, ok


@pytest.mark.parametrize("filt", ["hardware", "exact"])
def test_raycast_volume_full_config0(pkg, device, oracle, filt):
    """Config 0 at its full size: 128^3 blob volume, 512x512, with the
    texture unit's trilinear filter (default, as the reference's CUDA device)
    and with the exact fp32 filter of the CPU device."""
    sc = pkg.scenes.config0()
    sc["renderer"]["volumeFilter"] = filt
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    good, frac = raycast_ok(gpu, F)
    assert good, f"only {frac:.5f} of pixels within {RAYCAST_TOL}"
    assert np.all(gpu["depth"] == np.float32(1e31)) and np.all(F.depth == np.float32(1e31))
    assert np.all(gpu["normal"] == 0) and np.all(gpu["albedo"] == 0)
    assert gpu["errorFlags"] == 0
    assert gpu["color"][..., :3].max() > 0.05  # the volume is visible
    if filt == "exact":
        assert float(np.abs(gpu["color"] - F.color).max()) < 1e-4


def test_raycast_volume_sampling_rates(pkg, device, oracle):
    for rate in (0.5, 1.0, 3.0):
        sc = pkg.scenes.config0(res=96, n=40)
        sc["renderer"]["volumeSamplingRate"] = rate
        gpu = render_gpu(pkg, device, sc)
        _, F = render_oracle(oracle, sc)
        good, frac = raycast_ok(gpu, F)
        assert good, (rate, frac)


def small_spheres(pkg, res=128, spp=4, n=24, renderer="pathtrace", bounce=5, seed=None):
    kw = {} if seed is None else {"seed": seed}
    sc = pkg.scenes.config1(res=res, spp=spp, num_spheres=n, nu=24, nv=12, max_bounce=bounce, **kw)
    sc["renderer"]["type"] = renderer
    return sc


def test_raycast_triangles(pkg, device, oracle):
    sc = small_spheres(pkg, res=192, renderer="raycast")
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    good, frac = raycast_ok(gpu, F)
    assert good, frac
    hit = (F.depth < 1e30) & (gpu["depth"] < 1e30)
    assert hit.mean() > 0.2
    assert np.array_equal(F.depth < 1e30, gpu["depth"] < 1e30) or \
        (np.mean((F.depth < 1e30) != (gpu["depth"] < 1e30)) < 1e-3)
    rel = np.abs(gpu["depth"][hit] - F.depth[hit]) / F.depth[hit]
    assert float((rel <= 1e-4).mean()) >= 0.999
    nd = np.abs(gpu["normal"] - F.normal).max(axis=-1)
    assert float((nd <= 1e-3).mean()) >= 0.999
    ad = np.abs(gpu["albedo"] - F.albedo).max(axis=-1)
    assert float((ad <= 1e-5).mean()) >= 0.999


def gl_matrices(eye, target, up, fovy, aspect, near=0.5, far=500.0):
    """OpenGL-style view and projection matrices, column-major (the layout of
    the matrix camera's 'view' and 'proj' parameters)."""
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = s, u, -f
    view[:3, 3] = -view[:3, :3] @ eye
    t = 1.0 / np.tan(fovy / 2)
    proj = np.zeros((4, 4))
    proj[0, 0], proj[1, 1] = t / aspect, t
    proj[2, 2], proj[2, 3] = (far + near) / (near - far), 2 * far * near / (near - far)
    proj[3, 2] = -1.0
    return [float(v) for v in view.T.reshape(-1)], [float(v) for v in proj.T.reshape(-1)]


@pytest.mark.parametrize("kind", ["orthographic", "omnidirectional", "matrix"])
def test_raycast_camera_types(pkg, device, oracle, kind):
    """The orthographic, omnidirectional and matrix cameras (DeviceCopyableObjects.h
    :2510-2600) against the oracle's, through the raycast renderer."""
    sc = small_spheres(pkg, res=128, renderer="raycast")
    cam = dict(sc["camera"], type=kind)
    if kind == "orthographic":
        cam["height"] = 24.0
    elif kind == "omnidirectional":
        cam["position"] = [0.0, 2.0, 0.0]
    else:
        eye = np.asarray(cam["position"])
        view, proj = gl_matrices(eye, eye + np.asarray(cam["direction"]), cam["up"],
                                 cam["fovy"], 1.0)
        cam["view"], cam["proj"] = view, proj
    sc["camera"] = cam
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    good, frac = raycast_ok(gpu, F)
    hit = F.depth < 1e30
    print(kind, "within tolerance", frac, "hit share", float(hit.mean()))
    assert hit.mean() > 0.05
    assert good, frac


@pytest.mark.parametrize("wavefront", [True, False])
def test_pathtrace_same_stream(pkg, device, oracle, wavefront):
    """Same seeds: the GPU path tracer follows the oracle sample for sample,
    in both execution modes (wavefront queues / one thread per pixel)."""
    sc = small_spheres(pkg, res=128, spp=8)
    sc["renderer"]["wavefront"] = wavefront
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert not np.isnan(gpu["color"]).any()
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.97, float((d <= 1e-3).mean())
    hit = (F.depth < 1e30) & (gpu["depth"] < 1e30)
    rel = np.abs(gpu["depth"][hit] - F.depth[hit]) / F.depth[hit]
    assert float((rel <= 1e-4).mean()) >= 0.99
    assert gpu["errorFlags"] == 0


def test_pathtrace_statistical_band(pkg, device, oracle):
    """Independent streams: GPU mean within the combined 3-sigma band.

    The GPU's per-pixel variance comes from its own frames (each frame is a
    16-spp estimate; the accumulation buffer gives the running mean), the
    oracle's from its per-sample sums; sigma of the difference combines both.
    """
    frames, spp = 16, 16
    sc = small_spheres(pkg, res=64, spp=spp, n=16)
    h = pkg.scenes.build(device, sc)
    prev = None
    frame_means = []
    for k in range(frames):
        device.render(h["frame"])
        device.wait(h["frame"])
        acc = device.map(h["frame"], "channel.color")[..., :3].astype(np.float64)
        frame_means.append(acc if prev is None else (k + 1) * acc - k * prev)
        prev = acc
    gpu_mean = prev
    fm = np.stack(frame_means)
    var_gpu_mean = fm.var(axis=0, ddof=1) / frames
    # oracle with accumulation IDs 1000.. (independent LCG seeds)
    S, F = render_oracle(oracle, sc, frames=frames, accum_start=1000, stats=True)
    n = frames * spp
    mean = F.sum / n
    var = np.maximum(F.sumsq / n - mean * mean, 0.0) * n / (n - 1)
    sigma = np.sqrt(var_gpu_mean + var / n)
    inside = np.abs(gpu_mean - mean) <= 3.0 * sigma + 1e-6
    frac = float(inside.all(axis=-1).mean())
    rmse = float(np.sqrt(np.mean((gpu_mean - mean) ** 2)))
    print(f"3-sigma band: {frac:.4f} of pixels, RMSE {rmse:.5f}")
    assert frac >= 0.985, frac
    assert abs(float(gpu_mean.mean() - mean.mean())) < 0.01


def test_pathtrace_accumulation(pkg, device, oracle):
    """Progressive accumulation over frames (frame/Frame.cpp running mean)."""
    sc = small_spheres(pkg, res=64, spp=2, n=12)
    gpu = render_gpu(pkg, device, sc, frames=4)
    _, F = render_oracle(oracle, sc, frames=4)
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.97


def test_clip_plane(pkg, device, oracle):
    sc = small_spheres(pkg, res=128, renderer="raycast")
    sc["renderer"]["clipPlanes"] = [[0.0, 0.0, 1.0, 0.0]]
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    good, frac = raycast_ok(gpu, F)
    assert good, frac
    sc["renderer"]["type"] = "pathtrace"
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.97


def test_instance_transform(pkg, device, oracle):
    """A group placed by an instance transform (rotation + scale + translation)."""
    base = small_spheres(pkg, res=128, renderer="raycast", n=10)
    c, s = np.cos(0.4), np.sin(0.4)
    xfm = [c * 1.2, 0.0, -s * 1.2, 0.0, 1.2, 0.0, s * 1.2, 0.0, c * 1.2, 1.0, -0.5, 2.0]
    sc = dict(base)
    sc["instances"] = [{"transform": xfm, "surfaces": base["surfaces"][:5]}]
    sc["surfaces"] = base["surfaces"][5:]
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    good, frac = raycast_ok(gpu, F)
    assert good, frac


def test_color_formats(pkg, device, oracle):
    sc = pkg.scenes.config0(res=64, n=32)
    h = pkg.scenes.build(device, sc, channels=("depth",))
    vsr = pkg.vsr
    for t in (vsr.UFIXED8_VEC4, vsr.UFIXED8_RGBA_SRGB):
        device.set(h["frame"], "channel.color", t, vsr.DATA_TYPE)
        device.commit(h["frame"])
        device.render(h["frame"])
        device.wait(h["frame"])
        px = device.map(h["frame"], "channel.color")
        _, F = render_oracle(oracle, sc)
        c = np.clip(F.color, 0, 1)
        if t == vsr.UFIXED8_RGBA_SRGB:
            lin = c[..., :3]
            c[..., :3] = np.where(lin <= 0.0031308, 12.92 * lin, 1.055 * lin ** (1 / 2.4) - 0.055)
        ref = (255.0 * c).astype(np.uint32)
        got = np.stack([(px >> (8 * k)) & 255 for k in range(4)], -1)
        assert np.abs(got.astype(np.int64) - ref).max() <= 1


def test_incomplete_frame_reports_error(pkg, device):
    vsr = pkg.vsr
    f = device.frame()
    device.set(f, "size", (8, 8), vsr.UINT32_VEC2)
    device.commit(f)
    n0 = len(device.messages)
    assert device.render(f) == 6  # VSR_ERROR_INCOMPLETE
    assert any("incomplete" in m[2] for m in device.messages[n0:])
    device.release(f)


@pytest.mark.parametrize("chunks", [1, 8])
def test_full_config1_rows_against_oracle(pkg, device, oracle, chunks):
    """Config 1 at full size on the GPU; a band of rows checked against the
    oracle (chunks 8: the benchmark's setting)."""
    sc = pkg.scenes.config1()
    sc["renderer"]["sampleChunks"] = chunks
    h = pkg.scenes.build(device, sc)
    device.render(h["frame"])
    device.wait(h["frame"])
    color = device.map(h["frame"], "channel.color")
    assert device.get_uint(h["frame"], "errorFlags") == 0
    assert not np.isnan(color).any()
    S = oracle.Scene(sc)
    F = oracle.Frame(1024, 1024)
    oracle.render(S, F, rows=(500, 504))
    d = np.abs(color[500:504, :, :3] - F.color[500:504, :, :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.95


def small_volume_scene(pkg, res=64, spp=4, n=40, spheres=8):
    sc = pkg.scenes.config2(res=(res, res), spp=spp, n=n, num_spheres=spheres, nu=16, nv=8)
    sc["volumes"][0]["majorantBrickSize"] = 8
    return sc


@pytest.mark.parametrize("wavefront", [True, False])
def test_volume_pathtrace_same_stream(pkg, device, oracle, wavefront):
    """Delta tracking through the brick-majorant DDA: same stream as the oracle."""
    sc = small_volume_scene(pkg)
    sc["renderer"]["wavefront"] = wavefront
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc, grid=oracle.GRID_BRICK)
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.95, float((d <= 1e-3).mean())


def test_volume_pathtrace_unbiased_vs_unit_majorant(pkg, device, oracle):
    """Brick majorants vs the reference CUDA path's majorant of 1 (no grid):
    different random streams, same expectation (delta tracking is unbiased
    for any majorant that bounds the extinction)."""
    frames, spp = 8, 16
    sc = small_volume_scene(pkg, res=48, spp=spp)
    h = pkg.scenes.build(device, sc)
    prev, fms = None, []
    for k in range(frames):
        device.render(h["frame"])
        device.wait(h["frame"])
        acc = device.map(h["frame"], "channel.color")[..., :3].astype(np.float64)
        fms.append(acc if prev is None else (k + 1) * acc - k * prev)
        prev = acc
    var_gpu = np.stack(fms).var(axis=0, ddof=1) / frames
    S, F = render_oracle(oracle, sc, frames=frames, accum_start=500, stats=True,
                         grid=oracle.GRID_NONE)
    n = frames * spp
    mean = F.sum / n
    var = np.maximum(F.sumsq / n - mean * mean, 0.0) * n / (n - 1)
    inside = np.abs(prev - mean) <= 3.0 * np.sqrt(var_gpu + var / n) + 1e-6
    frac = float(inside.all(axis=-1).mean())
    print(f"volume 3-sigma band: {frac:.4f}")
    assert frac >= 0.98, frac


def gradient_volume_scene(pkg, res=96, n=48):
    """The config-0 blob volume lit by a directional light, with gradient
    shading on."""
    sc = pkg.scenes.config0(res=res, n=n)
    d = np.array([-0.35, -1.0, -0.45])
    d /= np.linalg.norm(d)
    sc["lights"] = [{"direction": [float(x) for x in d], "color": [1.0, 1.0, 1.0],
                     "irradiance": 2.5}]
    sc["renderer"].update(gradientShading=True, ambientRadiance=0.2)
    return sc


@pytest.mark.parametrize("filt", ["exact", "hardware"])
def test_raycast_gradient_shading(pkg, device, oracle, filt):
    """Raycast volume samples lit along the normalised central-difference
    field gradient (rayMarchVolume<1>), against the oracle's fp32 filter:
    the raycast bar with either filter (the texture unit's 8-bit filter
    weights move the gradient's direction slightly), and fp32 rounding only
    with the exact filter."""
    sc = gradient_volume_scene(pkg)
    sc["renderer"]["volumeFilter"] = filt
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    _, P = render_oracle(oracle, dict(sc, renderer=dict(sc["renderer"], gradientShading=False)))
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    # the shading changes the image
    assert np.abs(F.color[..., :3] - P.color[..., :3]).max() > 0.2 * P.color[..., :3].max()
    d = np.abs(gpu["color"] - F.color).max(axis=-1)
    print(filt, "within 2e-3:", float((d <= 2e-3).mean()), "max", float(d.max()))
    good, frac = raycast_ok(gpu, F)
    assert good, frac
    if filt == "exact":
        assert float(d.max()) < 1e-4


@pytest.mark.parametrize("wavefront", [False, True])
def test_volume_pathtrace_gradient_shading_same_stream(pkg, device, oracle, wavefront):
    """Path-traced scatter events shaded as a matte surface along the field
    gradient at the hit (Pathtrace_impl.cpp:203-212, 313-328), same random
    stream as the oracle; a wavefront renderer hands such frames to the
    megakernel."""
    sc = small_volume_scene(pkg)
    sc["renderer"].update(gradientShading=True, volumeFilter="exact", wavefront=wavefront)
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc, grid=oracle.GRID_BRICK)
    _, P = render_oracle(oracle, dict(sc, renderer=dict(sc["renderer"], gradientShading=False)),
                         grid=oracle.GRID_BRICK)
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    assert float(np.abs(F.color[..., :3] - P.color[..., :3]).mean()) > 1e-3
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.95, float((d <= 1e-3).mean())


def point_and_spot_lights():
    """A point light above the sphere set and a spot aimed at its centre."""
    spot_pos = np.array([4.0, 14.0, 10.0])
    axis = np.array([0.0, -1.0, 0.0]) - spot_pos
    axis /= np.linalg.norm(axis)
    return [{"type": "point", "position": [0.0, 12.0, 5.0], "intensity": 300.0,
             "color": [1.0, 0.9, 0.8]},
            {"type": "spot", "position": spot_pos.tolist(), "direction": axis.tolist(),
             "openingAngle": 0.6, "falloffAngle": 0.15, "intensity": 400.0,
             "color": [0.7, 0.8, 1.0]}]


def test_raycast_point_and_spot_lights(pkg, device, oracle):
    """Point and spot lights (sampleLight towards the hit point, inverse-square
    falloff, the spot's smoothstep cone) in the raycast renderer."""
    sc = small_spheres(pkg, res=128, renderer="raycast")
    sc["lights"] = point_and_spot_lights()
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    _, P = render_oracle(oracle, dict(sc, lights=sc["lights"][:1]))
    assert gpu["errorFlags"] == 0
    assert float(np.abs(F.color - P.color).max()) > 0.05  # the spot lights part of the view
    good, frac = raycast_ok(gpu, F)
    assert good, frac


@pytest.mark.parametrize("wavefront", [True, False])
def test_pathtrace_point_and_spot_same_stream(pkg, device, oracle, wavefront):
    """Next-event estimation towards point and spot lights (three draws per
    light sample, shadow rays ending at the light), same stream as the
    oracle, in both execution modes."""
    sc = small_spheres(pkg, res=96, spp=8)
    sc["lights"] = point_and_spot_lights()
    sc["renderer"]["wavefront"] = wavefront
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.97, float((d <= 1e-3).mean())


def test_instanced_lights(pkg, device, oracle):
    """Lights inside an instanced group: positions by the instance's affine
    transform, directions by its linear part (xfmLight)."""
    base = small_spheres(pkg, res=96, renderer="raycast", n=10)
    c, s = np.cos(0.4), np.sin(0.4)
    xfm = [c * 1.2, 0.0, -s * 1.2, 0.0, 1.2, 0.0, s * 1.2, 0.0, c * 1.2, 1.0, -0.5, 2.0]
    sc = dict(base)
    sc["lights"] = []
    sc["instances"] = [{"transform": xfm, "surfaces": base["surfaces"][:5],
                        "lights": point_and_spot_lights() + base["lights"]}]
    sc["surfaces"] = base["surfaces"][5:]
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    good, frac = raycast_ok(gpu, F)
    assert good, frac


def test_volume_pathtrace_point_light_gradient_shading(pkg, device, oracle):
    """A point light inside the config-2 style volume with gradient shading:
    scatter events lit towards the light, same stream as the oracle."""
    sc = small_volume_scene(pkg)
    sc["lights"] = [{"type": "point", "position": [2.0, 6.0, 4.0], "intensity": 200.0}]
    sc["renderer"].update(gradientShading=True, volumeFilter="exact")
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc, grid=oracle.GRID_BRICK)
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.95, float((d <= 1e-3).mean())


def sphere_surfaces(base, n=40, seed=3):
    """Two sphere geometries over the sphere-set volume: one with per-sphere
    radii, one placed through primitive.index; the materials of the first
    two surfaces of `base`."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-10.0, 10.0, (n, 3)).astype(np.float32)
    radii = rng.uniform(0.3, 1.5, n).astype(np.float32)
    h = n // 2
    return [{"geometry": "sphere", "vertices": centres[:h], "radii": radii[:h],
             "material": base["surfaces"][0]["material"]},
            {"geometry": "sphere", "vertices": centres, "indices": np.arange(h, n, dtype=np.uint32),
             "radii": radii[h:], "material": base["surfaces"][1]["material"]}]


def cone_cylinder_surfaces(base, n=16, seed=4):
    """A cone geometry (index pairs, radii per vertex) and a cylinder
    geometry (consecutive end points, radius per cylinder) over the
    sphere-set volume."""
    rng = np.random.default_rng(seed)

    def segments():
        a = rng.uniform(-9.0, 9.0, (n, 3)).astype(np.float32)
        b = (a + rng.uniform(-3.0, 3.0, (n, 3))).astype(np.float32)
        return np.stack([a, b], axis=1).reshape(-1, 3)

    # separate end points: a cone and a cylinder on one axis would share
    # coplanar cap discs, whose order at equal t is a coin toss
    cone_ends, cyl_ends = segments(), segments()
    return [{"geometry": "cone", "vertices": cone_ends,
             "indices": np.arange(2 * n, dtype=np.uint32).reshape(-1, 2)[::-1].copy(),
             "radii": rng.uniform(0.2, 1.2, 2 * n).astype(np.float32),
             "material": base["surfaces"][2]["material"]},
            {"geometry": "cylinder", "vertices": cyl_ends,
             "radii": rng.uniform(0.2, 0.8, n).astype(np.float32),
             "material": base["surfaces"][3]["material"]}]


def quad_surfaces(base, n=24, seed=6, flat=False):
    """Planar quads of random orientation and size over the sphere-set
    volume, half through primitive.index (as UINT32_VEC4), half as
    consecutive vertices; each quad k is shaded with the normal of
    tessellated triangle k, i.e. mostly another quad's. flat: horizontal
    quads facing up, for which that normal is each quad's own."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-9.0, 9.0, (n, 3))
    u = rng.normal(size=(n, 3))
    w = rng.normal(size=(n, 3))
    if flat:
        u[:, 1] = 0.0
        w = np.cross(np.array([0.0, 1.0, 0.0]), u)
    u *= rng.uniform(0.8, 2.5, (n, 1)) / np.linalg.norm(u, axis=1, keepdims=True)
    w -= (w * u).sum(1, keepdims=True) * u / (u * u).sum(1, keepdims=True)
    w *= rng.uniform(0.8, 2.5, (n, 1)) / np.linalg.norm(w, axis=1, keepdims=True)
    v = np.stack([c - u - w, c + u - w, c + u + w, c - u + w], axis=1).astype(np.float32)
    h = n // 2
    second = v[h:].reshape(-1, 3)[::-1].copy()
    order = np.arange(4 * (n - h), dtype=np.uint32).reshape(-1, 4)[:, ::-1]
    if flat:  # keep the winding (and so the facing) of the second half
        second = v[h:].reshape(-1, 3).copy()
        order = np.arange(4 * (n - h), dtype=np.uint32).reshape(-1, 4)
    return [{"geometry": "quad", "vertices": v[:h].reshape(-1, 3),
             "material": base["surfaces"][0]["material"]},
            {"geometry": "quad", "vertices": second, "indices": order.copy(),
             "material": base["surfaces"][1]["material"]}]


@pytest.mark.parametrize("kinds", ["spheres", "cones_cylinders", "quads"])
def test_raycast_analytic_primitives(pkg, device, oracle, kinds):
    """Spheres, cones and cylinders (their own BVH per group, each kind's
    intersection and normal), and quads (two triangles each, the reference's
    normal rule) beside triangle meshes, raycast."""
    sc = small_spheres(pkg, res=128, renderer="raycast")
    extra = {"spheres": sphere_surfaces, "cones_cylinders": cone_cylinder_surfaces,
             "quads": quad_surfaces}[kinds](sc)
    sc["surfaces"] = sc["surfaces"] + extra
    sc["lights"] = sc["lights"] + point_and_spot_lights()[:1]
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    good, frac = raycast_ok(gpu, F)
    assert good, frac
    hit = (F.depth < 1e30) & (gpu["depth"] < 1e30)
    rel = np.abs(gpu["depth"][hit] - F.depth[hit]) / F.depth[hit]
    assert float((rel <= 1e-4).mean()) >= 0.999
    nd = np.abs(gpu["normal"] - F.normal).max(axis=-1)
    assert float((nd <= 1e-3).mean()) >= 0.999
    # the spheres are in view: the image differs from the one without them
    _, P = render_oracle(oracle, dict(sc, surfaces=sc["surfaces"][:-2]))
    assert float((np.abs(F.color - P.color).max(axis=-1) > 1e-3).mean()) > 0.02


@pytest.mark.parametrize("wavefront", [True, False])
def test_pathtrace_analytic_primitives_same_stream(pkg, device, oracle, wavefront):
    """Path tracing over spheres, cones, cylinders and triangles with the
    same stream as the oracle (a wavefront renderer hands such worlds to the
    megakernel)."""
    sc = small_spheres(pkg, res=96, spp=8)
    sc["surfaces"] = sc["surfaces"] + sphere_surfaces(sc) + cone_cylinder_surfaces(sc)
    sc["renderer"]["wavefront"] = wavefront
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.97, float((d <= 1e-3).mean())


def test_pathtrace_quads_same_stream(pkg, device, oracle):
    """Path tracing over quads and triangles, same stream as the oracle. The
    quads are horizontal and face one way, so the reference's normal rule
    (quad k shaded with triangle k's normal) gives each its own normal; with
    mixed orientations a quad can be shaded, and its bounce rays offset, along
    another quad's normal, so that rays start on the wrong side of their
    surface and self-hits turn on rounding (the raycast test covers that
    rule)."""
    sc = small_spheres(pkg, res=96, spp=8)
    sc["surfaces"] = sc["surfaces"] + quad_surfaces(sc, flat=True)
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.97, float((d <= 1e-3).mean())


def test_instanced_analytic_primitives(pkg, device, oracle):
    """A group of spheres, cones and cylinders placed by an instance
    transform (rotation, scale, translation), next to world-level triangles."""
    base = small_spheres(pkg, res=96, renderer="raycast", n=10)
    c, s = np.cos(0.4), np.sin(0.4)
    xfm = [c * 1.2, 0.0, -s * 1.2, 0.0, 1.2, 0.0, s * 1.2, 0.0, c * 1.2, 1.0, -0.5, 2.0]
    sc = dict(base)
    sc["instances"] = [{"transform": xfm,
                        "surfaces": sphere_surfaces(base, n=16) + cone_cylinder_surfaces(base, 8)}]
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    good, frac = raycast_ok(gpu, F)
    assert good, frac


def iso_surface(pkg, seed=7):
    """A two-level iso-surface of a 40^3 blob field over [-8,8]^3."""
    rng = np.random.default_rng(seed)
    return {"geometry": "isosurface", "data": pkg.scenes.blob_field(40, rng),
            "origin": [-8.0, -8.0, -8.0], "spacing": [16.0 / 39] * 3, "isovalues": [0.3, 0.6],
            "material": {"type": "matte", "color": [0.3, 0.7, 0.4]}}


def test_raycast_isosurface(pkg, device, oracle):
    """Iso-surfaces of a structured field (the lattice march and the
    gradient normal) beside triangle meshes, raycast."""
    sc = small_spheres(pkg, res=96, renderer="raycast")
    sc["surfaces"] = sc["surfaces"] + [iso_surface(pkg)]
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    good, frac = raycast_ok(gpu, F)
    assert good, frac
    hit = (F.depth < 1e30) & (gpu["depth"] < 1e30)
    rel = np.abs(gpu["depth"][hit] - F.depth[hit]) / F.depth[hit]
    assert float((rel <= 1e-4).mean()) >= 0.999


def test_pathtrace_isosurface_same_stream(pkg, device, oracle):
    """Path tracing over an iso-surface and triangles, same stream as the
    oracle."""
    sc = small_spheres(pkg, res=96, spp=8)
    sc["surfaces"] = sc["surfaces"] + [iso_surface(pkg)]
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.97, float((d <= 1e-3).mean())


def test_wavefront_equals_megakernel(pkg, device):
    """The two execution modes produce the same frame (same stream, same math)."""
    sc = small_spheres(pkg, res=96, spp=4, n=16)
    sc["renderer"]["wavefront"] = True
    a = render_gpu(pkg, device, sc, frames=2)
    sc["renderer"]["wavefront"] = False
    b = render_gpu(pkg, device, sc, frames=2)
    d = np.abs(a["color"] - b["color"]).max(axis=-1)
    assert float((d <= 1e-5).mean()) >= 0.99
    assert np.array_equal(a["depth"], b["depth"])


@pytest.mark.parametrize("build,width", [("fast", 2), ("quality", 4), ("fast", 4)])
def test_bvh_build_policies_give_the_same_image(pkg, device, build, width):
    """LBVH / PLOC builds and 2- / 4-wide nodes are different trees over the
    same triangles; closest hits are ordered by (t, instance, triangle), so
    every combination renders the frame of the default (PLOC, 2-wide)."""
    sc = small_spheres(pkg, res=96, spp=2, n=20)
    a = render_gpu(pkg, device, sc)
    sc["bvhBuild"], sc["bvhWidth"] = build, width
    b = render_gpu(pkg, device, sc)
    assert np.array_equal(a["depth"], b["depth"])
    d = np.abs(a["color"] - b["color"]).max(axis=-1)
    assert float((d <= 1e-6).mean()) >= 0.995


@pytest.mark.parametrize("leaf", [1, 2, 8, 32])
@pytest.mark.parametrize("build", ["quality", "fast"])
def test_bvh_leaf_sizes_give_the_same_image(pkg, device, build, leaf):
    """Leaves of up to `leaf` triangles (world parameter bvhLeafSize, the
    depth-first triangle order and relinked nodes of the leaf collapse)
    against the default leaf size: the same hits, so the same depth and,
    up to rare exact ties, the same colour, for both builders."""
    sc = small_spheres(pkg, res=96, spp=2, n=20)
    sc["bvhBuild"] = build
    a = render_gpu(pkg, device, sc)
    sc["bvhLeafSize"] = leaf
    b = render_gpu(pkg, device, sc)
    assert np.array_equal(a["depth"], b["depth"])
    assert np.array_equal(a["normal"], b["normal"])
    d = np.abs(a["color"] - b["color"]).max(axis=-1)
    assert float((d <= 1e-6).mean()) >= 0.995
    assert a["errorFlags"] == 0 and b["errorFlags"] == 0


def test_bvh_leaf_size_in_a_volume_world(pkg, device):
    """Worlds with volumes keep one triangle per leaf unless bvhLeafSize is
    set; set to 8 the same path-traced frame comes out (same hits, the same
    random stream through the delta tracking)."""
    sc = small_volume_scene(pkg, res=64, spp=4, spheres=12)
    a = render_gpu(pkg, device, sc)
    sc["bvhLeafSize"] = 8
    b = render_gpu(pkg, device, sc)
    assert np.array_equal(a["depth"], b["depth"])
    d = np.abs(a["color"] - b["color"]).max(axis=-1)
    assert float((d <= 1e-6).mean()) >= 0.995
    assert a["errorFlags"] == 0 and b["errorFlags"] == 0


def translucent_spheres(pkg, renderer, res=96, spp=8, n=16):
    """The sphere set with non-opaque materials: a third "blend" with opacity
    0.25..0.75, a third "mask" with opacity either side of its cutoff (0.5),
    the rest (and the ground) opaque, so that the stochastic-opacity loop
    (one draw per surface hit, re-trace past a rejected hit) and the
    closest-hit shadow rays of a non-opaque world both run."""
    sc = small_spheres(pkg, res=res, spp=spp, n=n, renderer=renderer)
    rng = np.random.default_rng(21)
    for k, s in enumerate(sc["surfaces"][:-1]):
        m = dict(s["material"])
        if k % 3 == 0:
            m.update(alphaMode="blend", opacity=float(rng.uniform(0.25, 0.75)))
        elif k % 3 == 1:
            m.update(alphaMode="mask", opacity=float(rng.choice([0.3, 0.7])), alphaCutoff=0.5)
        s["material"] = m
    return sc


def test_raycast_nonopaque_materials(pkg, device, oracle):
    """Raycast through blend / mask materials (surface layers composited
    front to back until alpha reaches 0.999, Raycast_impl.cpp:100-156)."""
    sc = translucent_spheres(pkg, "raycast", res=128)
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    opaque = {k: v for k, v in sc.items()}
    opaque["surfaces"] = [dict(s, material={kk: vv for kk, vv in s["material"].items()
                                            if kk not in ("alphaMode", "opacity", "alphaCutoff")})
                          for s in sc["surfaces"]]
    _, P = render_oracle(oracle, opaque)
    assert gpu["errorFlags"] == 0
    # the materials change the image
    assert float((np.abs(F.color - P.color).max(axis=-1) > 1e-2).mean()) > 0.02
    good, frac = raycast_ok(gpu, F)
    assert good, frac
    hit = (F.depth < 1e30) & (gpu["depth"] < 1e30)
    rel = np.abs(gpu["depth"][hit] - F.depth[hit]) / F.depth[hit]
    assert float((rel <= 1e-4).mean()) >= 0.999


@pytest.mark.parametrize("wavefront", [True, False])
def test_pathtrace_nonopaque_materials_same_stream(pkg, device, oracle, wavefront):
    """Stochastic opacity (intersectSurfaces<EvalOpacity>, renderer/common.h
    :1502-1543): a hit is rejected when a uniform draw exceeds the material's
    opacity and the ray is traced on from just past it; same stream as the
    oracle, in both execution modes."""
    sc = translucent_spheres(pkg, "pathtrace")
    sc["renderer"]["wavefront"] = wavefront
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    frac = float((d <= 1e-3).mean())
    print("non-opaque same-stream within 1e-3:", frac)
    assert frac >= 0.97, frac


def surfaces_and_volume(pkg, res=128, n=64, spheres=12):
    """A raycast world with triangle meshes inside a blob volume: the config-0
    field and transfer function over the sphere set's box [-12, 12]^3 (unit
    distance one voxel spacing), the config-1 camera."""
    sc = small_spheres(pkg, res=res, renderer="raycast", n=spheres)
    v = pkg.scenes.config0(res=32, n=n)["volumes"][0]
    spacing = 24.0 / (n - 1)
    v = dict(v, origin=[-12.0] * 3, spacing=[spacing] * 3, unitDistance=spacing)
    sc["volumes"] = [v]
    sc["renderer"]["volumeSamplingRate"] = 2.0
    return sc


@pytest.mark.parametrize("filt", ["hardware", "exact"])
def test_raycast_surfaces_and_volume(pkg, device, oracle, filt):
    """Raycast compositing with surfaces and a volume (Raycast_impl.cpp
    :158-240): the surface over the background, then the volume marched up
    to the surface hit and composited over that; a pixel whose ray meets the
    volume keeps the surface's depth but zero normal and albedo."""
    sc = surfaces_and_volume(pkg)
    sc["renderer"]["volumeFilter"] = filt
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    _, P = render_oracle(oracle, dict(sc, volumes=[]))
    assert gpu["errorFlags"] == 0
    assert float((np.abs(F.color - P.color).max(axis=-1) > 1e-2).mean()) > 0.1
    good, frac = raycast_ok(gpu, F)
    print(filt, "within 2e-3:", frac)
    assert good, frac
    hit = (F.depth < 1e30) & (gpu["depth"] < 1e30)
    assert hit.mean() > 0.1
    assert np.array_equal(F.depth < 1e30, gpu["depth"] < 1e30)
    rel = np.abs(gpu["depth"][hit] - F.depth[hit]) / F.depth[hit]
    assert float((rel <= 1e-4).mean()) >= 0.999
    assert np.array_equal(gpu["normal"] == 0, F.normal == 0)
    if filt == "exact":
        assert float(np.abs(gpu["color"] - F.color).max()) < 1e-3


@pytest.mark.parametrize("chunks", [1, 4])
def test_pathtrace_sample_chunks_same_stream(pkg, device, oracle, chunks):
    """Sample chunks: a frame's samples as `chunks` concurrent streams, each
    seeded and accumulated as a sub-frame (accumulation IDs chunks * accumID
    + c); over two frames the GPU follows the oracle, which renders the same
    sub-frames one after another."""
    sc = small_spheres(pkg, res=96, spp=8, n=16)
    sc["renderer"]["sampleChunks"] = chunks
    gpu = render_gpu(pkg, device, sc, frames=2)
    _, F = render_oracle(oracle, sc, frames=2)
    assert gpu["errorFlags"] == 0
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    frac = float((d <= 1e-3).mean())
    print(f"sample chunks {chunks}: {frac:.4f} of pixels within 1e-3")
    assert frac >= 0.97, frac
    hit = (F.depth < 1e30) & (gpu["depth"] < 1e30)
    rel = np.abs(gpu["depth"][hit] - F.depth[hit]) / F.depth[hit]
    assert float((rel <= 1e-4).mean()) >= 0.99
    if chunks > 1:  # the streams differ from the single-stream frame
        sc1 = dict(sc, renderer=dict(sc["renderer"], sampleChunks=1))
        _, F1 = render_oracle(oracle, sc1, frames=2)
        assert float(np.abs(F1.color - F.color).max()) > 1e-3


@pytest.mark.parametrize("chunks", [1, 8])
def test_pathtrace_1024spp_band_config1_scene(pkg, device, oracle, chunks):
    """The path-tracer bar: the config-1 scene (all 256 spheres, 64x32
    segments, ground quad, depth 5) at 128x128, 1024 spp on each side with
    independent random streams (GPU accumulation IDs 0..15, oracle 1000..).
    The GPU's 1024-spp mean must lie inside the 3-sigma band of the
    difference of the two means (sigma from the oracle's per-sample variance
    and the variance of the GPU's 16 frame means) on >= 98.5 % of pixels;
    the RMSE between the two means and the share inside the oracle's own
    3-sigma band are printed."""
    frames, spp = 16, 64
    sc = pkg.scenes.config1(res=128, spp=spp)
    sc["renderer"]["sampleChunks"] = chunks
    h = pkg.scenes.build(device, sc)
    prev, fms = None, []
    for k in range(frames):
        assert device.render(h["frame"]) == 0
        assert device.wait(h["frame"])
        acc = device.map(h["frame"], "channel.color")[..., :3].astype(np.float64)
        fms.append(acc if prev is None else (k + 1) * acc - k * prev)
        prev = acc
    assert device.get_uint(h["frame"], "errorFlags") == 0
    for o in (h["frame"], h["renderer"], h["camera"], h["world"], *h["keep"]):
        device.release(o)
    gpu_mean = prev
    var_gpu_mean = np.stack(fms).var(axis=0, ddof=1) / frames
    _, F = render_oracle(oracle, sc, frames=frames, accum_start=1000, stats=True, tile=16)
    n = frames * spp
    mean = F.sum / n
    var = np.maximum(F.sumsq / n - mean * mean, 0.0) * n / (n - 1)
    sigma_ref = np.sqrt(var / n)
    sigma = np.sqrt(var_gpu_mean + var / n)
    inside = float((np.abs(gpu_mean - mean) <= 3.0 * sigma + 1e-6).all(axis=-1).mean())
    inside_ref = float((np.abs(gpu_mean - mean) <= 3.0 * sigma_ref + 1e-6).all(axis=-1).mean())
    rmse = float(np.sqrt(np.mean((gpu_mean - mean) ** 2)))
    print(f"1024 spp, 128x128, {chunks} chunks: inside combined 3-sigma band {inside:.4f}, "
          f"inside the oracle's "
          f"own band {inside_ref:.4f}, RMSE {rmse:.5f}, mean {float(mean.mean()):.4f}")
    assert inside >= 0.985, inside
    assert abs(float(gpu_mean.mean() - mean.mean())) < 0.01 * float(mean.mean()) + 1e-3


def config2_oracle(oracle, sc, lib=None, rows=None, frames=1, accum_start=0, stats=False):
    """The oracle's frame of a config-2 style scene (brick majorants), from
    the plain build or from the library at `lib` (e.g. the contracted one)."""
    saved = (oracle.LIB_PATH, oracle._lib)
    try:
        if lib:
            oracle.LIB_PATH, oracle._lib = lib, None
        S = oracle.Scene(sc, grid_method=oracle.GRID_BRICK)
        W, H = sc["frame"]["size"]
        F = oracle.Frame(W, H, stats=stats)
        F.f.accumID = accum_start
        for _ in range(frames):
            oracle.render(S, F, rows=rows, tile=16)
        S.close()
        return F
    finally:
        oracle.LIB_PATH, oracle._lib = saved


def render_frames_gpu(pkg, device, sc, frames):
    """Accumulate `frames` frames; the accumulated colour and each frame's
    own mean (for the variance of the GPU mean)."""
    h = pkg.scenes.build(device, sc)
    prev, fms = None, []
    for k in range(frames):
        assert device.render(h["frame"]) == 0
        assert device.wait(h["frame"])
        acc = device.map(h["frame"], "channel.color")[..., :3].astype(np.float64)
        fms.append(acc if prev is None else (k + 1) * acc - k * prev)
        prev = acc
    err = device.get_uint(h["frame"], "errorFlags")
    for o in (h["frame"], h["renderer"], h["camera"], h["world"], *h["keep"]):
        device.release(o)
    return prev, np.stack(fms), err


@pytest.mark.parametrize("case", ["band", "crop"])
def test_volume_pathtrace_config2_settings_same_stream(pkg, device, oracle, contracted, case):
    """Config 2 at its own settings: the 512^3 value-noise field with the
    default 16^3-voxel brick majorants (32^3 bricks walked by the DDA), the
    clip plane (0,0,1,0), depth 8, the config-1 spheres; same random stream
    as the oracle at 4 spp. band: the full 1920x1080 frame on the GPU, rows
    538..541 against the oracle; crop: a 256x256 frame of the same world.

    This world is rounding-sensitive: thousands of tracking steps per path
    (density scale 50), each a comparison of a sampled value with a random
    draw, so a last-bit difference sends a sample down another path. The
    bar is therefore relative: the GPU must agree with the oracle (within
    1e-3 per pixel) at least as well, less 5 points, as the oracle built
    with multiply-add contraction does; the means must agree."""
    spp = 4
    if case == "band":
        sc = pkg.scenes.config2(spp=spp)
        rows = (538, 542)
    else:
        sc = pkg.scenes.config2(res=(256, 256), spp=spp)
        rows = None
    assert sc["volumes"][0]["majorantBrickSize"] == 16
    assert sc["renderer"]["clipPlanes"] == [[0.0, 0.0, 1.0, 0.0]]
    color, _, err = render_frames_gpu(pkg, device, sc, 1)
    assert err == 0
    assert not np.isnan(color).any()
    W, H = sc["frame"]["size"]
    r0, r1 = rows if rows else (0, H)
    o = config2_oracle(oracle, sc, rows=rows).color[r0:r1, :, :3]
    c = config2_oracle(oracle, sc, lib=contracted, rows=rows).color[r0:r1, :, :3]
    g = color[r0:r1]
    assert float(o.max()) > 0.05  # the band sees the volume and the spheres
    gpu_frac = float((np.abs(g - o).max(axis=-1) <= 1e-3).mean())
    fma_frac = float((np.abs(c - o).max(axis=-1) <= 1e-3).mean())
    print(f"config2 {case}, {spp} spp: GPU vs oracle {gpu_frac:.4f} of pixels within 1e-3, "
          f"contracted oracle vs oracle {fma_frac:.4f}")
    assert gpu_frac >= fma_frac - 0.05, (gpu_frac, fma_frac)
    assert abs(float(g.mean()) - float(o.mean())) < 0.03 * float(o.mean()) + 2e-3


def test_volume_pathtrace_config2_statistical_band(pkg, device, oracle):
    """Config 2's world (512^3 field, 16^3 bricks, clip plane, depth 8, the
    spheres) as a 128x128 frame, 256 spp on each side with independent
    streams (GPU 16 frames of 16 spp, oracle accumulation IDs 1000..): the
    GPU mean lies inside the 3-sigma band of the difference of the two means
    on >= 98 % of pixels (sigma from the oracle's per-sample variance and the
    variance of the GPU's frame means); RMSE printed."""
    frames, spp = 16, 16
    sc = pkg.scenes.config2(res=(128, 128), spp=spp)
    gpu_mean, fms, err = render_frames_gpu(pkg, device, sc, frames)
    assert err == 0
    var_gpu = fms.var(axis=0, ddof=1) / frames
    F = config2_oracle(oracle, sc, frames=frames, accum_start=1000, stats=True)
    n = frames * spp
    mean = F.sum / n
    var = np.maximum(F.sumsq / n - mean * mean, 0.0) * n / (n - 1)
    sigma = np.sqrt(var_gpu + var / n)
    inside = float((np.abs(gpu_mean - mean) <= 3.0 * sigma + 1e-6).all(axis=-1).mean())
    rmse = float(np.sqrt(np.mean((gpu_mean - mean) ** 2)))
    print(f"config2 128x128, 256 spp: inside the 3-sigma band {inside:.4f}, RMSE {rmse:.5f}, "
          f"mean {float(mean.mean()):.4f} (GPU {float(gpu_mean.mean()):.4f})")
    assert inside >= 0.98, inside
    assert abs(float(gpu_mean.mean() - mean.mean())) < 0.02 * float(mean.mean()) + 1e-3


@pytest.mark.parametrize("wavefront", [False, True])
def test_sample_mask_renders_only_masked_pixels(pkg, device, oracle, wavefront):
    """vsrFrameSampleMask: one frame over every pixel, then frames under two
    different masks (a checkerboard, then its top half with one more
    stripe). Each pixel's mean is the mean of the frames that rendered it
    (the oracle's single frames with the same accumulation IDs, i.e. the
    same streams), and pixels outside every mask keep the first frame."""
    import torch
    sc = small_spheres(pkg, res=64, spp=2, n=12)
    sc["renderer"]["wavefront"] = wavefront
    h = pkg.scenes.build(device, sc)
    yy, xx = np.mgrid[0:64, 0:64]
    checker = (((xx // 4) + (yy // 4)) % 2).astype(np.uint8)
    second = ((checker.astype(bool) & (yy < 32)) | ((xx // 4) % 4 == 1)).astype(np.uint8)
    masks = [None, checker, checker, second]
    keep = []
    for m in masks:
        if m is None:
            device.sample_mask(h["frame"], None)
        else:
            t = torch.from_numpy(m.reshape(-1)).cuda()
            keep.append(t)
            device.sample_mask(h["frame"], t.data_ptr())
        assert device.render(h["frame"]) == 0
        assert device.wait(h["frame"])
    got = device.map(h["frame"], "channel.color")[..., :3]
    assert device.get_uint(h["frame"], "errorFlags") == 0
    device.sample_mask(h["frame"], None)
    for o in (h["frame"], h["renderer"], h["camera"], h["world"], *h["keep"]):
        device.release(o)
    # each frame's own mean (sum of its samples / spp) at accumulation ID k
    single = [render_oracle(oracle, sc, accum_start=k, stats=True)[1].sum / 2.0 for k in range(4)]
    num = np.zeros((64, 64, 3))
    cnt = np.zeros((64, 64, 1))
    for k, m in enumerate(masks):
        on = np.ones((64, 64), bool) if m is None else m.astype(bool)
        num[on] += single[k][on]
        cnt[on] += 1
    expect = num / cnt
    d = np.abs(got - expect).max(axis=-1)
    frac = float((d <= 1e-3).mean())
    print("sample mask: within 1e-3 of the per-pixel frame mean:", frac)
    assert frac >= 0.97, frac
    untouched = cnt[..., 0] == 1
    assert untouched.any() and (cnt[..., 0] == 2).any() and (cnt[..., 0] >= 3).any()
    assert float((d[untouched] <= 1e-3).mean()) >= 0.97


@pytest.mark.parametrize("move", [False, True])
def test_pathtrace_taa_same_stream(pkg, device, oracle, move):
    """Temporal anti-aliasing (renderer taa, taaAlpha; frame/Frame.cpp
    :339-381): each frame's own mean colour and motion vectors, then the
    resolve pass blends the reprojected previous result (cardinal-spline
    history read, albedo test). Four frames, with the camera still (the
    frames accumulate seeds, motion vectors are zero) or moving sideways
    (each camera commit restarts accumulation but keeps the history); every
    frame's resolved colour follows the oracle's."""
    import ctypes
    sc = small_spheres(pkg, res=96, spp=4, n=16)
    sc["renderer"].update(taa=True, taaAlpha=0.3)
    h = pkg.scenes.build(device, sc)
    S = oracle.Scene(sc)
    F = oracle.Frame(96, 96, taa=True)
    cam = dict(sc["camera"])
    right = np.cross(np.asarray(cam["direction"]), np.asarray(cam["up"]))
    right /= np.linalg.norm(right)
    vsr = pkg.vsr
    try:
        for k in range(4):
            if move and k > 0:
                cam["position"] = [float(p + 0.4 * r) for p, r in zip(cam["position"], right)]
                device.set(h["camera"], "position", cam["position"], vsr.FLOAT32_VEC3)
                device.commit(h["camera"])
                S = oracle.Scene(dict(sc, camera=dict(cam)))
                oracle.load().or_frame_reset(ctypes.byref(F.f))
            assert device.render(h["frame"]) == 0
            assert device.wait(h["frame"])
            got = device.map(h["frame"], "channel.color")
            oracle.render(S, F)
            d = np.abs(got[..., :3] - F.color[..., :3]).max(axis=-1)
            frac = float((d <= 1e-3).mean())
            print(f"taa move={move} frame {k}: {frac:.4f} within 1e-3")
            assert frac >= 0.97, (k, frac)
        assert device.get_uint(h["frame"], "errorFlags") == 0
    finally:
        for o in (h["frame"], h["renderer"], h["camera"], h["world"], *h["keep"]):
            device.release(o)


def quad_lights(direct=True):
    """An invisible overhead quad light over the config-1 sphere set and a
    small visible one in the middle of the view (tilted, lit on both
    sides)."""
    return [{"type": "quad", "position": [-6.0, 14.0, -6.0], "edge1": [12.0, 0.0, 0.0],
             "edge2": [0.0, 0.0, 12.0], "intensity": 2.0, "color": [1.0, 0.95, 0.9],
             "visible": False},
            {"type": "quad", "position": [0.5, 1.0, 14.0], "edge1": [4.0, 0.0, 0.0],
             "edge2": [0.0, 3.0, 1.0], "intensity": 4.0, "color": [1.0, 0.8, 0.6]}]


def test_raycast_quad_lights(pkg, device, oracle):
    """Quad lights in the raycast renderer: each surface hit samples every
    light once with the zero-state stream (A |cos| / d^2 weighting); rays
    that leave the surfaces through a visible quad light show its intensity
    (Raycast_impl.cpp:158-172)."""
    sc = small_spheres(pkg, res=128, renderer="raycast")
    sc["lights"] = quad_lights() + sc["lights"]
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    seen = np.all(np.abs(F.color - np.array([4.0, 3.2, 2.4, 1.0], np.float32)) < 1e-6, axis=-1)
    assert 0.01 < float(seen.mean()) < 0.2  # the visible light covers part of the view
    good, frac = raycast_ok(gpu, F)
    assert good, frac


@pytest.mark.parametrize("wavefront", [True, False])
def test_pathtrace_quad_lights_same_stream(pkg, device, oracle, wavefront):
    """Quad lights in the path tracer (area sampling of one triangle of the
    quad, MIS weights on light samples and on BSDF-sampled rays that hit a
    light, a visible light ending camera paths), with a directional light
    beside them; the same stream as the oracle. Frames with quad lights run
    the megakernel in either execution mode."""
    sc = small_spheres(pkg, res=96, spp=8)
    sc["lights"] = quad_lights() + sc["lights"]
    sc["renderer"]["wavefront"] = wavefront
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.97, float((d <= 1e-3).mean())


def test_pathtrace_quad_light_mis_expectation(pkg, device):
    """The GPU's mean over 16 384 path-traced samples of a matte plane under
    an invisible unit quad light 2 above it lies within 5 sigma of the
    closed-form expectation of the reference's weighting (next-event
    estimation and BSDF-sampled hits, power heuristic, the light sample
    weighted against the BSDF sample drawn at the same hit)."""
    import math
    g = 50.0
    quad = np.array([[-g, -g, 0], [g, -g, 0], [g, g, 0], [-g, g, 0]], np.float32)
    sc = {
        "surfaces": [{"vertices": quad, "indices": np.array([[0, 1, 2], [0, 2, 3]], np.uint32),
                      "material": {"type": "matte", "color": [0.6, 0.5, 0.4]}}],
        "volumes": [],
        "lights": [{"type": "quad", "position": [-0.5, -0.5, 2.0], "edge1": [1.0, 0.0, 0.0],
                    "edge2": [0.0, 1.0, 0.0], "intensity": 3.0, "color": [1.0, 0.9, 0.8],
                    "visible": False}],
        "camera": {"type": "orthographic", "position": [0.0, 0.0, 10.0],
                   "direction": [0.0, 0.0, -1.0], "up": [0.0, 1.0, 0.0], "height": 0.01,
                   "aspect": 1.0},
        "renderer": {"type": "pathtrace", "pixelSamples": 64, "maxBounce": 3,
                     "ambientRadiance": 0.0, "ambientSamples": 0, "background": [0, 0, 0, 1]},
        "frame": {"size": (16, 16)},
    }
    gpu = render_gpu(pkg, device, sc)
    assert gpu["errorFlags"] == 0
    px = gpu["color"][..., :3].reshape(-1, 3).astype(np.float64)
    n = px.shape[0] * 64
    mean = px.mean(0)
    sigma = px.std(0) / math.sqrt(px.shape[0])  # per-pixel means of 64 samples
    k = 400
    t = (np.arange(k) + 0.5) / k - 0.5
    U, V = np.meshgrid(t, t)
    d = np.sqrt(U * U + V * V + 4.0)
    cos = 2.0 / d
    geo = cos * cos / (d * d)
    a2 = (math.pi / cos) ** 2
    w_nee = a2 * np.log1p(1.0 / a2)
    p_bsdf, p_hit = cos / math.pi, d * d / cos
    w_bsdf = p_bsdf ** 2 / (p_bsdf ** 2 + p_hit ** 2)
    expect = np.array([0.6, 0.5, 0.4]) / math.pi * 3.0 * np.array([1.0, 0.9, 0.8]) * \
        float((geo * (w_nee + w_bsdf)).mean())
    assert n == 16384
    assert np.all(np.abs(mean - expect) <= 5 * sigma + 1e-4 * expect), (mean, expect, sigma)


def hdri_light(visible=True, seed=7):
    """A 64 x 32 sky: a vertical gradient, seeded noise and a bright sun
    patch, scale 0.8, frame from up and direction."""
    rng = np.random.default_rng(seed)
    H, W = 32, 64
    v = (np.arange(H) + 0.5) / H
    img = np.empty((H, W, 3), np.float32)
    img[...] = (0.2 + 0.8 * (1 - v))[:, None, None] * np.array([0.5, 0.7, 1.0], np.float32)
    img *= rng.uniform(0.8, 1.2, size=(H, W, 1)).astype(np.float32)
    img[6:9, 20:24] = [40.0, 36.0, 30.0]
    return {"type": "hdri", "radiance": img, "scale": 0.8, "up": [0.0, 1.0, 0.2],
            "direction": [0.3, 0.0, 1.0], "visible": visible}


def test_raycast_hdri_light(pkg, device, oracle):
    """An HDRI light in the raycast renderer: each surface hit samples it
    once with the zero-state stream (CDF texel, toPolar direction, bilinear
    radiance), and rays that leave the surfaces show the sky
    (Raycast_impl.cpp:158-172)."""
    sc = small_spheres(pkg, res=128, renderer="raycast")
    sc["lights"] = [hdri_light()] + sc["lights"]
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    assert float((F.depth > 1e30).mean()) > 0.05  # part of the view is sky
    good, frac = raycast_ok(gpu, F)
    assert good, frac


@pytest.mark.parametrize("wavefront", [True, False])
def test_pathtrace_hdri_light_same_stream(pkg, device, oracle, wavefront):
    """An HDRI light beside a directional light in the path tracer (CDF
    sampling with the two draws in the reference CPU device's order, MIS
    against the BSDF sample, sky radiance for rays that leave the scene,
    its hit density for the BSDF sample's weight), same stream as the
    oracle, in either execution mode (HDRI frames run the megakernel)."""
    sc = small_spheres(pkg, res=96, spp=8)
    sc["lights"] = [hdri_light()] + sc["lights"]
    sc["renderer"]["wavefront"] = wavefront
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.97, float((d <= 1e-3).mean())


def test_pathtrace_hdri_expectation(pkg, device):
    """The GPU's mean over 16 384 samples of a matte plane under an HDRI
    whose only bright texels are row 2 of 8 lies within 5 sigma of the
    closed-form expectation of the reference's sampling (next-event
    estimation at the band's texel corner, BSDF samples through the
    bilinear band, both MIS-weighted as the reference weights them)."""
    import math
    W, H, y0, V, s_ = 16, 8, 2, 4.0, 1.5
    img = np.zeros((H, W, 3), np.float32)
    img[y0] = V
    g = 50.0
    quad = np.array([[-g, -g, 0], [g, -g, 0], [g, g, 0], [-g, g, 0]], np.float32)
    sc = {
        "surfaces": [{"vertices": quad, "indices": np.array([[0, 1, 2], [0, 2, 3]], np.uint32),
                      "material": {"type": "matte", "color": [0.6, 0.5, 0.4]}}],
        "volumes": [],
        "lights": [{"type": "hdri", "radiance": img, "scale": s_, "up": [0.0, 0.0, -1.0],
                    "direction": [1.0, 0.0, 0.0], "visible": False}],
        "camera": {"type": "orthographic", "position": [0.0, 0.0, 10.0],
                   "direction": [0.0, 0.0, -1.0], "up": [0.0, 1.0, 0.0], "height": 0.01,
                   "aspect": 1.0},
        "renderer": {"type": "pathtrace", "pixelSamples": 64, "maxBounce": 3,
                     "ambientRadiance": 0.0, "ambientSamples": 0, "background": [0, 0, 0, 1]},
        "frame": {"size": (16, 16)},
    }
    gpu = render_gpu(pkg, device, sc)
    assert gpu["errorFlags"] == 0
    px = gpu["color"][..., :3].reshape(-1, 3).astype(np.float64)
    mean = px.mean(0)
    sigma = px.std(0) / math.sqrt(px.shape[0])
    rho = np.array([0.6, 0.5, 0.4])
    a2 = (math.pi * H / (4 * math.pi)) ** 2
    e_nee = 2 * rho * V * s_ * math.cos(math.pi * y0 / H) / H * a2 * math.log1p(1 / a2)
    k = 200000
    th = (np.arange(k) + 0.5) / k * (math.pi / 2)
    v = np.clip(th / math.pi, 0.001, 0.999)
    yy = v * H - 0.5
    f0 = np.floor(yy)
    fy = yy - f0
    band = np.where(f0 == y0, 1 - fy, np.where(f0 + 1 == y0, fy, 0.0))
    p_b = np.cos(th) / math.pi
    p_l = H / (2 * math.pi ** 2 * np.sin(th))
    w = p_b ** 2 / (p_b ** 2 + p_l ** 2)
    integral = float((band * w * np.cos(th) / math.pi * 2 * math.pi * np.sin(th)).sum() *
                     (math.pi / 2) / k)
    expect = e_nee + rho * V * s_ * integral
    assert np.all(np.abs(mean - expect) <= 5 * sigma + 1e-4 * expect), (mean, expect, sigma)


@pytest.mark.parametrize("renderer", ["raycast", "pathtrace"])
def test_axis_parallel_rays(pkg, device, oracle, renderer):
    """Rays whose direction has exact zero components (an orthographic
    camera looking straight down -z, ray origins inside and on the x / y
    slabs of the plane's boxes): the slab test must not turn 0 x inf or
    inf - inf into NaN and miss every box."""
    g = 4.0
    quad = np.array([[-g, -g, 0], [g, -g, 0], [g, g, 0], [-g, g, 0]], np.float32)
    sc = {
        "surfaces": [{"vertices": quad, "indices": np.array([[0, 1, 2], [0, 2, 3]], np.uint32),
                      "material": {"type": "matte", "color": [0.6, 0.5, 0.4]}}],
        "volumes": [],
        "lights": [{"direction": [0.0, 0.0, -1.0], "irradiance": 2.0}],
        "camera": {"type": "orthographic", "position": [0.0, 0.0, 10.0],
                   "direction": [0.0, 0.0, -1.0], "up": [0.0, 1.0, 0.0], "height": 10.0,
                   "aspect": 1.0},
        "renderer": {"type": renderer, "pixelSamples": 1, "ambientRadiance": 0.2,
                     "background": [0.1, 0.2, 0.3, 1.0]},
        "frame": {"size": (20, 20)},
    }
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    hit = F.depth < 1e30
    assert 0.5 < float(hit.mean()) < 0.9  # the plane covers the middle of the view
    assert np.array_equal(gpu["depth"] < 1e30, hit)
    assert np.allclose(gpu["depth"][hit], 10.0, rtol=1e-5)
    d = np.abs(gpu["color"] - F.color).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.99, float((d <= 1e-3).mean())


def textured_spheres(pkg, res=96, spp=4, renderer="pathtrace"):
    """The config-1 sphere set with geometry attributes and samplers:
    smooth vertex normals on every sphere, vertex colours read through the
    "color" attribute on every second sphere, a roughness image1D sampler
    on attribute0 (the vertex height) on every third, and a nearest-filtered
    image2D checker repeated over the ground through per-vertex texture
    coordinates (attribute0)."""
    sc = small_spheres(pkg, res=res, spp=spp, renderer=renderer)
    rough = {"type": "image1D", "image": np.linspace(0.05, 0.95, 16, dtype=np.float32),
             "inAttribute": "attribute0", "filter": "linear"}
    for k, s in enumerate(sc["surfaces"][:-1]):
        v = np.asarray(s["vertices"], np.float32)
        c = v.mean(axis=0)
        n = (v - c) / np.linalg.norm(v - c, axis=1, keepdims=True)
        s["normals"] = n.astype(np.float32)
        h = ((v[:, 1] - v[:, 1].min()) / max(float(np.ptp(v[:, 1])), 1e-6)).astype(np.float32)
        s["attributes"] = {"attribute0": h}
        if k % 2 == 0:
            s["attributes"]["color"] = np.concatenate(
                [0.5 + 0.5 * n, np.ones((len(n), 1), np.float32)], axis=1).astype(np.float32)
            s["material"] = dict(s["material"])
            key = "color" if s["material"]["type"] == "matte" else "baseColor"
            s["material"][key] = "color"
        if k % 3 == 0 and s["material"]["type"] == "physicallyBased":
            s["material"] = dict(s["material"], roughness={"sampler": rough})
    ground = sc["surfaces"][-1]
    gv = np.asarray(ground["vertices"], np.float32)
    ground["attributes"] = {"attribute0": (gv[:, [0, 2]] / 8.0).astype(np.float32)}
    chk = np.indices((8, 8)).sum(axis=0) % 2
    img = np.where(chk[..., None] == 1, [0.9, 0.85, 0.8], [0.2, 0.25, 0.3]).astype(np.float32)
    ground["material"] = {"type": "matte", "color": {"sampler": {
        "type": "image2D", "image": img, "filter": "nearest", "wrapMode1": "repeat",
        "wrapMode2": "repeat"}}}
    return sc


def test_raycast_textured(pkg, device, oracle):
    """Geometry attributes, vertex normals and samplers in the raycast
    renderer (getAttributes, getNormals' vertex normals, image1D / image2D
    samplers, material parameters from attributes)."""
    sc = textured_spheres(pkg, res=128, renderer="raycast")
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    _, P = render_oracle(oracle, small_spheres(pkg, res=128, renderer="raycast"))
    assert gpu["errorFlags"] == 0
    assert float(np.abs(F.color - P.color).max()) > 0.1  # the attributes change the image
    good, frac = raycast_ok(gpu, F)
    assert good, frac
    ad = np.abs(gpu["albedo"] - F.albedo).max(axis=-1)
    assert float((ad <= 1e-4).mean()) >= 0.999


@pytest.mark.parametrize("wavefront", [True, False])
def test_pathtrace_textured_same_stream(pkg, device, oracle, wavefront):
    """The same world in the path tracer, same stream as the oracle (frames
    with attributes run the megakernel in either execution mode)."""
    sc = textured_spheres(pkg, res=96, spp=8)
    sc["renderer"]["wavefront"] = wavefront
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.97, float((d <= 1e-3).mean())


def hair_curves(seed=11, n=40):
    """Seeded cubic strands above the sphere set: n multi-segment curves
    (2 segments each through primitive.index), radii 0.08..0.2 per strand."""
    rng = np.random.default_rng(seed)
    verts, idx = [], []
    for k in range(n):
        p = rng.uniform(-9.0, 9.0, 3)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        pts = [p + d * 2.0 * j / 6.0 + rng.normal(scale=0.6, size=3) * (j % 3 != 0)
               for j in range(7)]
        idx.append(len(verts))
        verts += pts
    return {"geometry": "bezierCurve", "vertices": np.asarray(verts, np.float32),
            "indices": np.asarray(idx, np.uint32),
            "radii": rng.uniform(0.08, 0.2, n).astype(np.float32),
            "material": {"type": "physicallyBased", "baseColor": [0.8, 0.6, 0.3],
                         "metallic": 0.2, "roughness": 0.5}}


def test_raycast_bezier_curves(pkg, device, oracle):
    """Cubic Bezier curves (the Phantom ray-hair intersector, curve normals)
    beside the triangle spheres in the raycast renderer: colour, depth and
    normal parity."""
    sc = small_spheres(pkg, res=128, renderer="raycast")
    sc["surfaces"] = sc["surfaces"] + [hair_curves()]
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    _, P = render_oracle(oracle, small_spheres(pkg, res=128, renderer="raycast"))
    assert gpu["errorFlags"] == 0
    strands = (F.depth < P.depth - 1e-3)
    assert float(strands.mean()) > 0.02  # the strands cover part of the view
    good, frac = raycast_ok(gpu, F)
    assert good, frac
    hit = (F.depth < 1e30) & (gpu["depth"] < 1e30)
    rel = np.abs(gpu["depth"][hit] - F.depth[hit]) / F.depth[hit]
    assert float((rel <= 1e-4).mean()) >= 0.999


@pytest.mark.parametrize("wavefront", [True, False])
def test_pathtrace_bezier_curves_same_stream(pkg, device, oracle, wavefront):
    """The strands in the path tracer, same stream as the oracle (frames
    with analytic primitives run the megakernel)."""
    sc = small_spheres(pkg, res=96, spp=8)
    sc["surfaces"] = sc["surfaces"] + [hair_curves()]
    sc["renderer"]["wavefront"] = wavefront
    gpu = render_gpu(pkg, device, sc)
    _, F = render_oracle(oracle, sc)
    assert gpu["errorFlags"] == 0
    assert not np.isnan(gpu["color"]).any()
    d = np.abs(gpu["color"][..., :3] - F.color[..., :3]).max(axis=-1)
    assert float((d <= 1e-3).mean()) >= 0.97, float((d <= 1e-3).mean())


def test_raycast_volume_march_units_grow(pkg, device, oracle):
    """A blob volume filling a 192^2 view needs more segment work units than
    the frame's first unit list holds: the first frame marches the rays
    beyond it whole, the next one with the list grown to the first frame's
    need; both match the oracle at the raycast bar."""
    import math
    sc = pkg.scenes.config0(res=192, n=128)
    extent = 127.0
    view = np.array([0.6, 0.45, 0.66])
    view /= np.linalg.norm(view)
    eye = np.array([extent / 2] * 3) + 0.75 * math.sqrt(3.0) * extent * view
    sc["camera"] = pkg.scenes._look_at_camera([extent / 2] * 3, list(eye), 40.0, 1.0)
    _, F = render_oracle(oracle, sc)
    h = pkg.scenes.build(device, sc)
    try:
        caps = []
        for k in range(2):
            assert device.render(h["frame"]) == 0
            assert device.wait(h["frame"])
            gpu = {"color": device.map(h["frame"], "channel.color")}
            good, frac = raycast_ok(gpu, F)
            assert good, (k, frac)
            assert device.get_uint(h["frame"], "errorFlags") == 0
            caps.append((device.get_uint(h["frame"], "march.unitsNeeded"),
                         device.get_uint(h["frame"], "march.unitCapacity")))
        (need0, cap0), (need1, cap1) = caps
        assert need0 > cap0, caps  # the first frame's list was too short
        assert need1 == need0 and cap1 >= need1, caps
    finally:
        for o in (h["frame"], h["renderer"], h["camera"], h["world"]):
            device.release(o)
        for o in h["keep"]:
            device.release(o)
