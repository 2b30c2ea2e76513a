"""Learned texture decoder on the tensor cores against the CPU oracle (oracle/neural.py).

* decode: texels decoded by the inference kernel equal the oracle's forward pass after unorm8
  quantisation, within one step (BF16 activations may round differently when the FP32 tensor-core
  sums or tanh.approx differ from the oracle's float64 by a rounding boundary);
* gradients: parameter and latent gradients of the training kernel for explicit samples within
  2e-3 relative (L2) of the oracle's backward pass on the same BF16 operands;
* training: the loss falls; the texture levels decoded 1:1 from their latent level come back
  within a few unorm8 steps, and the magnified levels 0 and 1 beat the plain texture at the
  latent grid's resolution (texture level 2) magnified bilinearly by at least 2 dB of PSNR;
* bounded waits: a wait that nothing completes returns SWR_ETIMEOUT and leaves the context usable;
* resolve: with a model whose network outputs each material's constant texel the neural resolve
  equals the plain resolve bit for bit (every pixel finds its decoded texels), and with a trained
  model its colours stay close to the plain resolve.
"""
import numpy as np
import pytest

from glimpsw_gb300 import scenes
from oracle import neural as N
from tests.helpers import GpuRenderer, default_lights, gpu_lights

pytestmark = pytest.mark.gpu

SIZE = 128
LEVELS = 4             # latent levels
DECODED = LEVELS + 2   # texture levels 0 .. 5 are decoded


def _device_texture(layers, size=SIZE):
    from glimpsw_gb300 import api
    t = api.Texture2D(api.FORMAT_RGBA8U, size, size, 16, len(layers))
    for i, px in enumerate(layers):
        t.set_pixels(np.ascontiguousarray(px, dtype=np.uint32), i)
    t.generate_mips()
    return t


class Plain:
    """Host copy of a device texture's storage for target lookups."""

    def __init__(self, t):
        self.t = t
        self.data = t.get_data()
        self.row_shift = int(np.log2(max(t.width, 8)))

    def targets(self, level, x, y):
        a0, a1 = N.plain_texels(self.data, self.row_shift, self.t.mip_offsets, self.t.layer_stride, self.t.num_layers,
                                level, x, y)
        return N.targets_from_words(a0, a1)


def _random_texels(rng, n, levels=range(DECODED), size=SIZE):
    levels = np.asarray(list(levels))
    w = 2.0 ** -levels.astype(np.float64)
    lvl = rng.choice(levels, n, p=w / w.sum())
    return lvl, rng.integers(0, size >> lvl), rng.integers(0, size >> lvl)


def _taps(m, lvl, x, y):
    return N.latent_taps(lvl, x, y, [s[0] for s in m.level_size], [s[1] for s in m.level_size], m.level_offset)


def _decode(m, mat, lvl, x, y):
    import torch
    from glimpsw_gb300 import api
    packed = api.pack_texel(lvl, x, y).astype(np.uint32)
    dt = torch.from_numpy(packed.view(np.int32)).cuda()
    out = torch.zeros(2 * len(packed), dtype=torch.int32, device="cuda")
    m.decode(mat, dt, len(packed), out)
    w = out.cpu().numpy().view(np.uint32).reshape(-1, 2)
    ch = [w[:, 0] & 255, (w[:, 0] >> 8) & 255, (w[:, 0] >> 16) & 255, w[:, 1] & 255, (w[:, 1] >> 8) & 255,
          (w[:, 1] >> 16) & 255, w[:, 1] >> 24, w[:, 0] >> 24]
    return np.stack(ch, axis=-1).astype(np.int64)


def _setup_stream():
    import torch
    from glimpsw_gb300 import api
    api.load_library()
    api.set_stream(torch.cuda.current_stream().cuda_stream)
    return api


@pytest.fixture(scope="module")
def model():
    api = _setup_stream()
    texs = [_device_texture([scenes.value_noise_rgba(SIZE, 11 + i, cells=8, layer=l, detail=True) for l in range(2)])
            for i in range(4)]
    m = api.NeuralMaterials(texs, latent_levels=LEVELS, seed=5)
    return m, texs, [Plain(t) for t in texs]


def test_model_layout_and_memory(model):
    m, texs, _ = model
    assert m.level_size == [(32, 32), (16, 16), (8, 8), (4, 4)]
    assert m.level_offset == [0, 1024, 1280, 1344] and m.texels_per_material == 1360
    mem = m.memory()
    assert mem["latent_bytes"] == 4 * 1360 * 16
    assert mem["plain_bytes"] == 4 * texs[0].layer_stride * 4 * 2
    # a 128^2 texture has levels 128..4 (6 levels), all decoded: nothing is left for the plain sampler
    assert texs[0].mip_levels == DECODED and mem["fallback_bytes"] == 0
    # latent level k starts as texture level k + 2, mapped to [-1, 1]
    p = Plain(texs[0])
    lat = m.get_latents(0)
    assert np.allclose(lat[5 * 32 + 3, :7], p.targets(np.array([2]), np.array([3]), np.array([5]))[0, :7] * 2 - 1, atol=1e-6)
    assert np.allclose(lat[1024 + 7 * 16 + 2, :7], p.targets(np.array([3]), np.array([2]), np.array([7]))[0, :7] * 2 - 1,
                       atol=1e-6)
    assert lat[5 * 32 + 3, 7] == 0


def _check_decode(m, seed=1, mat=2):
    """Random latents and parameters for one material, then 3000 texels of every decoded level:
    the inference kernel against the oracle's forward pass."""
    rng = np.random.default_rng(seed)
    lat = rng.normal(0, 0.8, (m.texels_per_material, 8)).astype(np.float32)
    m.set_latents(mat, lat)
    params = m.get_params(mat)
    params[N.PB2:N.PW3] = rng.normal(0, 0.2, 64)
    params[N.PW1:N.PW2].reshape(64, 16)[:, 9:11] = rng.normal(0, 0.5, (64, 2))
    m.set_params(mat, params)
    lvl, x, y = _random_texels(rng, 3000)
    got = _decode(m, mat, lvl, x, y)
    idx, fx, fy = _taps(m, lvl, x, y)
    exp = N.quantize(N.forward(params, N.latent_inputs(lat, idx, fx, fy), lvl)["y"])
    diff = np.abs(got - exp)
    print(f"decode: max |diff| {diff.max()}, differing outputs {(diff > 0).mean():.5f}")
    assert diff.max() <= 1 and (diff > 0).mean() < 0.05
    assert len(np.unique(exp[:, 0])) > 20  # the check is not vacuous
    for l in range(DECODED):
        assert (lvl == l).sum() > 10


def test_decode_matches_oracle(model):
    _check_decode(model[0])


def test_bounded_wait_times_out_and_context_stays_usable(model):
    """A device wait that nothing completes (an mbarrier armed for a copy that is never issued,
    with TMEM held) gives up at its limit and the call returns SWR_ETIMEOUT; the CTA frees its
    TMEM and exits, so the next kernels run normally: a decode with a host-set wait limit still
    matches the oracle."""
    api = _setup_stream()
    lib = api.load_library()
    for limit_ns in (1000, 1, 2_000_000):
        st = lib.swr_selftest_bounded_wait(limit_ns)
        assert st == api.SWR_ETIMEOUT, lib.swr_last_error().decode()
        assert "gave up" in lib.swr_last_error().decode()
    assert lib.swr_selftest_bounded_wait(0) == api.SWR_EINVAL
    m = model[0]
    with pytest.raises(Exception):
        m.set_wait_limit(0)
    m.set_wait_limit(50_000_000)  # 50 ms per wait
    try:
        _check_decode(m, seed=3)
    finally:
        m.set_wait_limit(1_000_000_000)


def test_gradients_match_oracle(model):
    import torch
    from glimpsw_gb300 import api
    m, _, plains = model
    rng = np.random.default_rng(2)
    mat = 1
    lat = rng.normal(0, 0.8, (m.texels_per_material, 8)).astype(np.float32)
    m.set_latents(mat, lat)
    params = m.get_params(mat)
    params[N.PB2:N.PW3] = rng.normal(0, 0.2, 64)
    params[N.PW1:N.PW2].reshape(64, 16)[:, 9:11] = rng.normal(0, 0.5, (64, 2))
    m.set_params(mat, params)
    n = 640
    lvl, x, y = _random_texels(rng, n)
    packed = api.pack_texel(lvl, x, y).astype(np.uint32)
    pg, lg, loss = m.gradients(mat, torch.from_numpy(packed.view(np.int32)).cuda(), n)
    idx, fx, fy = _taps(m, lvl, x, y)
    cache = N.forward(params, N.latent_inputs(lat, idx, fx, fy), lvl)
    g, dx0, l = N.backward(params, cache, plains[mat].targets(lvl, x, y))
    lgo = N.latent_gradient(dx0, idx, fx, fy, m.texels_per_material)
    assert abs(loss - l) <= 1e-3 * l
    blocks = {"W1": (slice(N.PW1, N.PW2), lambda a: a.reshape(64, 16)[:, :11]), "W2": (slice(N.PW2, N.PB2), None),
              "b2": (slice(N.PB2, N.PW3), None), "W3": (slice(N.PW3, N.PB3), None), "b3": (slice(N.PB3, N.PARAMS), None),
              "W1 level flags": (slice(N.PW1, N.PW2), lambda a: a.reshape(64, 16)[:, 9:11])}
    for name, (sl, view) in blocks.items():
        a, b = pg[sl].astype(np.float64), g[sl]
        if view:
            a, b = view(a), view(b)
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        print(f"{name}: rel L2 error {rel:.2e}")
        assert rel < 2e-3, name
    assert np.all(pg[N.PW1:N.PW2].reshape(64, 16)[:, 11:] == 0)
    rel = np.linalg.norm(lg - lgo) / np.linalg.norm(lgo)
    print(f"latent: rel L2 error {rel:.2e}")
    assert rel < 2e-3
    assert np.count_nonzero(np.abs(lgo).sum(1)) == np.count_nonzero(np.abs(lg).sum(1))


def _psnr_decoded(m, plains, rng, levels, n=4096):
    out = []
    for mat, p in enumerate(plains):
        lvl, x, y = _random_texels(rng, n, levels)
        got = _decode(m, mat, lvl, x, y)[:, :7] / 255.0
        out.append(N.psnr(got, p.targets(lvl, x, y)[:, :7]))
    return float(np.mean(out))


def _psnr_magnified(m, plains, rng, n=4096):
    """Without the network: texture level 2 (the latent grid's resolution) bilinearly magnified to
    levels 0 and 1 at the same taps, rounded to unorm8."""
    out = []
    for p in plains:
        lvl, x, y = _random_texels(rng, n, (0, 1))
        idx, fx, fy = _taps(m, lvl, x, y)
        LW = m.level_size[0][0]
        corners = [p.targets(np.full(n, 2), idx[:, k] % LW, idx[:, k] // LW)[:, :7] for k in range(4)]
        w = N.bilinear_weights(fx, fy)
        v = sum(w[:, k:k + 1] * corners[k] for k in range(4))
        out.append(N.psnr(np.rint(v * 255) / 255, p.targets(lvl, x, y)[:, :7]))
    return float(np.mean(out))


def test_training_decodes_and_beats_plain_magnification():
    api = _setup_stream()
    texs = [_device_texture([scenes.value_noise_rgba(SIZE, 31 + i, cells=8, layer=l, detail=True) for l in range(2)])
            for i in range(4)]
    plains = [Plain(t) for t in texs]
    m = api.NeuralMaterials(texs, latent_levels=LEVELS, seed=9)
    rng = np.random.default_rng(4)
    before = _psnr_decoded(m, plains, rng, range(DECODED))
    loss0 = m.train(1, batch=8192, materials_per_step=4, want_loss=True)
    m.train(3000, batch=8192, materials_per_step=4)
    loss1 = m.train(1, batch=8192, materials_per_step=4, want_loss=True)
    one_to_one = _psnr_decoded(m, plains, rng, range(2, DECODED))
    magnified = _psnr_decoded(m, plains, rng, (0, 1))
    base = _psnr_magnified(m, plains, rng)
    print(f"training: loss {loss0:.5f} -> {loss1:.5f}; PSNR untrained {before:.2f} dB; trained: levels 2-5 "
          f"{one_to_one:.2f} dB, levels 0-1 {magnified:.2f} dB vs plain level 2 magnified {base:.2f} dB")
    assert loss1 < 0.25 * loss0
    assert one_to_one > 40.0
    assert magnified > base + 2.0


def test_resolve_neural_constant_materials_equal_plain():
    """Each material's texture is one colour per layer and its network outputs that colour
    (W3 = 0, b3 = texel / 255): every decoded texel equals the plain one, so the neural resolve must
    reproduce the plain resolve exactly."""
    api = _setup_stream()
    sc = scenes.volume_scene(n=3000, width=320, height=180, n_materials=4, extent=25.0, texture_size=SIZE, env_size=64)
    rng = np.random.default_rng(6)
    cols = rng.integers(0, 256, (4, 2, 4)).astype(np.uint32)
    cols[:, 0, 3] = 255
    words = cols[..., 0] | (cols[..., 1] << 8) | (cols[..., 2] << 16) | (cols[..., 3] << 24)
    texs = [_device_texture([np.full((SIZE, SIZE), words[i, l], np.uint32) for l in range(2)]) for i in range(4)]
    m = api.NeuralMaterials(texs, latent_levels=LEVELS, seed=3)
    for i in range(4):
        p = np.zeros(N.PARAMS, np.float32)
        p[N.PB3:N.PARAMS] = np.concatenate([cols[i, 0, :3], cols[i, 1, :4], [255]]) / np.float32(255.0)
        m.set_params(i, p)
    g = GpuRenderer(sc.meshlets, sc.materials, texs)
    v = sc.views[0]
    lights = gpu_lights(default_lights())
    ctx = api.ShadingContext(g.scene, v.world_to_clip, world_to_clip=v.world_to_clip, view_pos=v.eye, lights=lights)
    a, _ = g.render(v.world_to_clip, v.width, v.height)
    b, _ = g.render(v.world_to_clip, v.width, v.height)
    ctx.resolve(g.rast, a)
    requests, tiles, per_level = ctx.resolve_neural(g.rast, b, m, want_stats=True)
    assert sum(per_level) == requests
    pa, pb = a.get_pixels(0), b.get_pixels(0)
    print(f"constant materials: {requests} decoded texels in {tiles} tiles (per level {per_level}), "
          f"{(pa != pb).sum()} pixels differ")
    assert requests > 1000 and tiles >= requests // 128
    assert np.array_equal(pa, pb)


def test_resolve_neural_close_to_plain():
    api = _setup_stream()
    sc = scenes.volume_scene(n=3000, width=320, height=180, n_materials=4, extent=25.0, texture_size=SIZE, env_size=64)
    # the benchmark materials' frequency content: 64-texel base cells plus the 8-texel detail octave
    texs = [_device_texture([scenes.value_noise_rgba(SIZE, 51 + i, cells=SIZE // 64, layer=l, detail=True)
                             for l in range(2)]) for i in range(4)]
    m = api.NeuralMaterials(texs, latent_levels=LEVELS, seed=3)
    m.train(3000, batch=8192, materials_per_step=4)
    g = GpuRenderer(sc.meshlets, sc.materials, texs)
    v = sc.views[0]
    ctx = api.ShadingContext(g.scene, v.world_to_clip, world_to_clip=v.world_to_clip, view_pos=v.eye,
                             lights=gpu_lights(default_lights()))
    a, _ = g.render(v.world_to_clip, v.width, v.height)
    b, _ = g.render(v.world_to_clip, v.width, v.height)
    ctx.resolve(g.rast, a)
    requests, _, per_level = ctx.resolve_neural(g.rast, b, m, want_stats=True)
    pa = a.get_pixels(0).view(np.uint8).reshape(v.height, v.width, 4)[..., :3] / 255.0
    pb = b.get_pixels(0).view(np.uint8).reshape(v.height, v.width, 4)[..., :3] / 255.0
    p = N.psnr(pa, pb)
    print(f"neural resolve: {requests} decoded texels (per level {per_level}), PSNR {p:.2f} dB, "
          f"max abs {np.abs(pa - pb).max() * 255:.0f}/255")
    assert requests > 1000
    assert p > 38.0


def test_checkpoint_save_load_resumes_training():
    """swr_neural_save / swr_neural_load: the restored model's checkpoint is byte-identical to the
    saved one, and training resumed from it follows the original model's trajectory. The latent
    gradient accumulates with float atomics, whose order varies from run to run, so the two
    continuations agree to a tolerance (rel. L2 1e-3 of parameters and latents) rather than bit for
    bit; a model trained the same number of steps from scratch lands far away."""
    api = _setup_stream()
    texs = [_device_texture([scenes.value_noise_rgba(SIZE, 41 + i, cells=8, layer=l, detail=True) for l in range(2)])
            for i in range(4)]
    a = api.NeuralMaterials(texs, latent_levels=LEVELS, seed=3)
    a.train(300, batch=8192, materials_per_step=4)
    blob = a.save()
    b = api.NeuralMaterials(texs, latent_levels=LEVELS, seed=99)
    b.load(blob)
    assert b.save() == blob
    fresh = api.NeuralMaterials(texs, latent_levels=LEVELS, seed=3)
    la = a.train(200, batch=8192, materials_per_step=4, want_loss=True)
    lb = b.train(200, batch=8192, materials_per_step=4, want_loss=True)
    lf = fresh.train(200, batch=8192, materials_per_step=4, want_loss=True)
    for mat in range(4):
        pa, pb, pf = a.get_params(mat), b.get_params(mat), fresh.get_params(mat)
        xa, xb = a.get_latents(mat), b.get_latents(mat)
        rel_p = np.linalg.norm(pa - pb) / np.linalg.norm(pa)
        rel_x = np.linalg.norm(xa - xb) / np.linalg.norm(xa)
        print(f"material {mat}: resumed vs continued rel L2 params {rel_p:.2e}, latents {rel_x:.2e}; "
              f"fresh {np.linalg.norm(pa - pf) / np.linalg.norm(pa):.2e}")
        assert rel_p < 1e-3 and rel_x < 1e-3
        assert np.linalg.norm(pa - pf) / np.linalg.norm(pa) > 1e-2
    assert abs(la - lb) <= 0.05 * la and lf > la
    # a checkpoint of a model of another shape is refused
    other = api.NeuralMaterials(texs[:2], latent_levels=LEVELS, seed=3)
    with pytest.raises(Exception):
        other.load(blob)
