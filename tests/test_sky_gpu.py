"""GPU parity of ocean_sky_envmap (the sky environment cube map) against the
FP32 oracle, which the CPU tests pin bit-exactly to the reference's own sky
shaders.  Tolerance: per texel |gpu - oracle| <= 1e-5 * (1 + |oracle|) (CUDA's
atanf / powf against the C library's), rel L2 < 1e-6 over the map; at most two
texels on the sun disk's rim may flip."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402
from test_sky_oracle import _assert_close, _oracle_map  # noqa: E402


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _gpu_map(torch, og, prm, S, tr, ins):
    dev = torch.device("cuda")
    t_tr = torch.from_numpy(np.ascontiguousarray(tr)).to(dev)
    t_ins = torch.from_numpy(np.ascontiguousarray(ins)).to(dev)
    out = torch.empty((6, S, S, 4), device=dev)
    og.sky_envmap(prm[0:3], prm[3:6], t_tr, t_ins, out, earth_pos=prm[6:9], beta_r=prm[9:12], mie_g=float(prm[12]),
                  sun_intensity=float(prm[13]))
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("case", [c["name"] for c in make_golden.SKY_CASES])
def test_sky_envmap_matches_oracle(torch_cuda, ocean_lib, oracle_mod, case):
    c = next(x for x in make_golden.SKY_CASES if x["name"] == case)
    tr, ins = make_golden.sky_tables(c["seed"])
    prm = make_golden.sky_prm(c)
    got = _gpu_map(torch_cuda, ocean_lib, prm, c["S"], tr, ins)
    _assert_close(got, _oracle_map(oracle_mod, prm, c["S"], tr, ins))
    # and the committed reference map
    g = np.load(os.path.join(HERE, "golden", "ref_sky.npz"))
    _assert_close(got, g[case])


def test_sky_envmap_full_size(torch_cuda, ocean_lib, oracle_mod):
    """The reference's 512 x 512 faces (ENVIRONMENT_MAP_SIZE, main.cpp:19)."""
    tr, ins = make_golden.sky_tables(21)
    prm = make_golden.sky_prm(dict(camera=(12.0, 25.0, -7.0), angle=-0.25))
    _assert_close(_gpu_map(torch_cuda, ocean_lib, prm, 512, tr, ins), _oracle_map(oracle_mod, prm, 512, tr, ins))


def test_sky_feeds_shading(torch_cuda, ocean_lib, oracle_mod):
    """The cube map from ocean_sky_envmap is the sky ocean_shade_grid reads."""
    torch = torch_cuda
    dev = torch.device("cuda")
    tr, ins = make_golden.sky_tables(3)
    sun = ocean_lib.sky_sun_direction(-0.35)
    prm = make_golden.sky_prm(dict(camera=(0.0, 10.0, 0.0), angle=-0.35))
    sky = torch.empty((6, 64, 64, 4), device=dev)
    ocean_lib.sky_envmap((0.0, 10.0, 0.0), sun, torch.from_numpy(tr).to(dev), torch.from_numpy(ins).to(dev), sky)
    rng = np.random.default_rng(4)
    n = 4096
    v = np.zeros((n, 8), np.float32)
    v[:, 0:3] = rng.uniform(-50, 50, (n, 3))
    nrm = rng.normal(size=(n, 3)) + np.array([0, 4.0, 0])
    v[:, 3:6] = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    colors = torch.empty((n, 4), device=dev)
    sea = (0.0, 0.2, 0.3)
    ocean_lib.shade_grid(torch.from_numpy(v).to(dev), (0.0, 10.0, 0.0), sun, sea, sky, colors)
    torch.cuda.synchronize()
    want = oracle_mod.shade(v.astype(np.float64), (0.0, 10.0, 0.0), sun, sea,
                            _oracle_map(oracle_mod, prm, 64, tr, ins).astype(np.float64))
    assert np.allclose(colors.cpu().numpy(), want, rtol=1e-4, atol=1e-5)


def test_sky_envmap_argument_errors(torch_cuda, ocean_lib):
    torch = torch_cuda
    dev = torch.device("cuda")
    tr = torch.zeros((64, 256, 4), device=dev)
    ins = torch.zeros((32, 128, 256, 4), device=dev)
    out = torch.empty((6, 8, 8, 4), device=dev)
    sun = ocean_lib.sky_sun_direction(-0.3)
    with pytest.raises(ocean_lib.OceanError):
        ocean_lib.sky_envmap((0.0, float("nan"), 0.0), sun, tr, ins, out)
    with pytest.raises(ocean_lib.OceanError):
        ocean_lib.sky_envmap((0.0, 1.0, 0.0), sun, tr, ins, torch.empty((6, 0, 0, 4), device=dev))
    flat = torch.zeros(6 * 8 * 8 * 4 + 1, device=dev)
    with pytest.raises(ocean_lib.OceanError):
        ocean_lib.sky_envmap((0.0, 1.0, 0.0), sun, tr, ins, flat[1:].view(6, 8, 8, 4))
    with pytest.raises(ocean_lib.OceanError):
        ocean_lib.sky_envmap((0.0, 1.0, 0.0), sun, tr, ins, out, beta_r=(0.0, 1e-5, 1e-5))
    ocean_lib.sky_envmap((0.0, 1.0, 0.0), sun, tr, ins, out)
    torch.cuda.synchronize()
    assert torch.isfinite(out).all()


@pytest.mark.parametrize("cam", [0, 1])
def test_skybox_matches_oracle(torch_cuda, ocean_lib, oracle_mod, cam):
    """ocean_render_skybox of a sky from ocean_sky_envmap against orc_skybox
    on the same cube map (FP32 against FP64: rtol 1e-4)."""
    from test_sky_oracle import SKYBOX_CAMERAS, look_at, perspective
    torch = torch_cuda
    dev = torch.device("cuda")
    eye, center, up, fovy = SKYBOX_CAMERAS[cam]
    W, H = 160, 96
    tr, ins = make_golden.sky_tables(8)
    sky = torch.empty((6, 128, 128, 4), device=dev)
    ocean_lib.sky_envmap(eye, ocean_lib.sky_sun_direction(-0.3), torch.from_numpy(tr).to(dev),
                         torch.from_numpy(ins).to(dev), sky)
    V, P = look_at(eye, center, up), perspective(fovy, W / H, 0.1, 1000.0)
    img = torch.empty((H, W, 4), device=dev)
    ocean_lib.render_skybox(sky, V.astype(np.float32), P.astype(np.float32), img)
    torch.cuda.synchronize()
    want = oracle_mod.skybox(sky.cpu().numpy().astype(np.float64), V.astype(np.float32), P.astype(np.float32), W, H)
    assert np.allclose(img.cpu().numpy(), want, rtol=1e-4, atol=1e-5)


def test_skybox_argument_errors(torch_cuda, ocean_lib):
    torch = torch_cuda
    dev = torch.device("cuda")
    sky = torch.zeros((6, 8, 8, 4), device=dev)
    img = torch.empty((4, 4, 4), device=dev)
    eye = np.eye(4, dtype=np.float32)
    with pytest.raises(ocean_lib.OceanError):
        ocean_lib.render_skybox(sky, eye, np.zeros((4, 4), np.float32), img)      # singular
    with pytest.raises(ocean_lib.OceanError):
        ocean_lib.render_skybox(sky, eye, eye, torch.empty((0, 4, 4), device=dev))
    ocean_lib.render_skybox(sky, eye, eye, img)
    torch.cuda.synchronize()
    assert torch.all(img[..., 3] == 1.0)
