"""The library's own FFT pipeline (spectral.cu): the padded-row R2C/C2R
against torch.fft (cuFFT), and the fused force pipeline against the cuFFT
path and the oracle."""
import numpy as np
import pytest
import torch

from oracle import cic, fourier
from conftest import rel_l2

pytestmark = pytest.mark.gpu

SHAPES = [(64, 64, 64), (8, 64, 16), (32, 128, 256), (128, 64, 32), (8, 256, 64), (8, 256, 256),
          (8, 512, 256), (8, 256, 512), (16, 512, 512)]


@pytest.fixture(params=["fused", "own"])
def fft_fused(lib, request):
    """The two library FFT paths of the composite calls: cuFFT planes around
    the fused x kernel, and the library's plane kernels as well."""
    from jaxpm_gb300 import distributed
    prev = distributed.set_fft_path(request.param)
    yield request.param
    distributed.set_fft_path(prev)


def r2c(x, batch=1):
    from jaxpm_gb300 import _lib
    nx, ny, nz = x.shape[-3:]
    pitch = _lib.load().pmgb_fft3_pitch(nz)
    out = torch.empty((batch, nx, ny, pitch), dtype=torch.complex64, device=x.device)
    _lib.call("pmgb_fft3_r2c_f32", _lib.ptr(x), _lib.ptr(out), nx, ny, nz, batch, _lib.stream())
    return out


def c2r(spec, nz, batch=1):
    from jaxpm_gb300 import _lib
    nx, ny = spec.shape[-3:-1]
    out = torch.empty((batch, nx, ny, nz), dtype=torch.float32, device=spec.device)
    _lib.call("pmgb_fft3_c2r_f32", _lib.ptr(spec), _lib.ptr(out), nx, ny, nz, batch,
              _lib.stream())
    return out


def test_supported_shapes(lib):
    assert lib.pmgb_fft3_supported(512, 512, 512) == 1
    assert lib.pmgb_fft3_supported(64, 64, 64) == 1
    assert lib.pmgb_fft3_supported(32, 32, 32) == 0    # ny below 64
    assert lib.pmgb_fft3_supported(48, 64, 64) == 0    # not a power of two
    assert lib.pmgb_fft3_supported(64, 1024, 64) == 0  # plane too large for one cluster
    assert lib.pmgb_fft3_pitch(512) == 264
    assert lib.pmgb_fft3_pitch(16) == 16


@pytest.mark.parametrize("shape", SHAPES)
def test_r2c_matches_cufft(cuda, fft_fused, shape):
    g = torch.Generator(device=cuda).manual_seed(1)
    x = torch.randn((2, *shape), device=cuda, generator=g)
    out = r2c(x, batch=2)
    nzh = shape[2] // 2 + 1
    ref = torch.fft.rfftn(x, dim=(1, 2, 3))
    got = out[..., :nzh]
    err = (got - ref).abs().max().item() / ref.abs().max().item()
    assert err < 2e-6, err
    assert torch.all(out[..., nzh:] == 0)


@pytest.mark.parametrize("shape", SHAPES)
def test_c2r_matches_cufft(cuda, fft_fused, shape):
    g = torch.Generator(device=cuda).manual_seed(2)
    x = torch.randn(shape, device=cuda, generator=g)
    spec = r2c(x)
    n = float(np.prod(shape))
    back = c2r(spec.clone(), shape[2])[0]
    assert rel_l2(back.cpu() / n, x.cpu()) < 1e-6
    # a spectrum made by cuFFT, padded
    ref = torch.fft.rfftn(x)
    padded = torch.zeros_like(spec[0])
    padded[..., :shape[2] // 2 + 1] = ref
    got = c2r(padded.unsqueeze(0), shape[2])[0]
    assert rel_l2(got.cpu(), (torch.fft.irfftn(ref, s=shape) * n).cpu()) < 1e-6


@pytest.mark.parametrize("shape", [(64, 64, 64), (32, 128, 64)])
def test_force_pipeline_matches_cufft_and_oracle(cuda, fft_fused, shape):
    """pm_forces through the fused spectral pipeline equals the cuFFT path
    and the float64 oracle."""
    from jaxpm_gb300 import distributed, pm
    rng = np.random.default_rng(4)
    n = int(np.prod(shape))
    lat = cic.lattice(shape).reshape(-1, 3)
    pos = (lat + rng.normal(0, 1.5, lat.shape)).astype(np.float32)
    x = torch.as_tensor(pos).to(cuda)
    f_auto = pm.pm_forces(x, shape, r_split=0.0).cpu()
    f_auto_rs = pm.pm_forces(x, shape, r_split=1.5).cpu()
    distributed.set_fft_path("cufft")
    f_cufft = pm.pm_forces(x, shape, r_split=0.0).cpu()
    f_cufft_rs = pm.pm_forces(x, shape, r_split=1.5).cpu()
    distributed.set_fft_path(fft_fused)
    # two float32 FFT implementations: rounding differences only
    assert rel_l2(f_auto, f_cufft) < 1e-5
    assert rel_l2(f_auto_rs, f_cufft_rs) < 1e-5
    ref = fourier.pm_forces(pos.astype(np.float64), shape, r_split=0.0, dtype=np.float64)
    assert rel_l2(f_auto.numpy(), ref) < 1e-5
    assert n == pos.shape[0]


def test_force_adjoint_matches_cufft(cuda, fft_fused):
    from jaxpm_gb300 import distributed, pm
    shape = (64, 64, 64)
    rng = np.random.default_rng(5)
    lat = cic.lattice(shape).reshape(-1, 3)
    pos = torch.as_tensor((lat + rng.normal(0, 1.0, lat.shape)).astype(np.float32)).to(cuda)
    g = torch.as_tensor(rng.standard_normal(lat.shape).astype(np.float32)).to(cuda)

    def grad():
        x = pos.clone().requires_grad_(True)
        (pm.pm_forces(x, shape) * g).sum().backward()
        return x.grad.cpu()

    a = grad()
    distributed.set_fft_path("cufft")
    b = grad()
    distributed.set_fft_path(fft_fused)
    assert rel_l2(a, b) < 1e-5


def test_sorted_run_spectral_matches_cufft(cuda, fft_fused):
    """Ten sorted-loop steps at 64^3 with the spectral pipeline against the
    same run through cuFFT, and the forward+adjoint through both."""
    from jaxpm_gb300 import cosmology, distributed, simulate
    shape = (64, 64, 64)
    rng = np.random.default_rng(6)
    lat = cic.lattice(shape).reshape(-1, 3)
    x0 = torch.as_tensor((lat + rng.normal(0, 0.5, lat.shape)).astype(np.float32)).to(cuda)
    v0 = torch.as_tensor(rng.normal(0, 0.2, lat.shape).astype(np.float32)).to(cuda)
    gx = torch.randn(x0.shape, device=cuda)
    gv = torch.randn(x0.shape, device=cuda)
    res = {}
    for path in (fft_fused, "cufft"):
        distributed.set_fft_path(path)
        eng = simulate.SortedFastPM(shape, cosmology.Planck15(), 0.1, 1.0, 10, device=cuda)
        eng.load(x0, v0)
        eng.run()
        xf, vf = eng.state()
        (_, _), (ax, av) = eng.vjp(x0, v0, gx, gv)
        res[path] = (xf.cpu(), vf.cpu(), ax.cpu(), av.cpu())
    distributed.set_fft_path(fft_fused)
    for a, b in zip(res[fft_fused], res["cufft"]):
        assert rel_l2(a, b) < 1e-4


@pytest.mark.parametrize("shape", [(64, 64, 64), (16, 64, 32), (32, 128, 256), (64, 256, 64)])
@pytest.mark.parametrize("r_split", [0.0, 1.5])
def test_mesh_forces_match_oracle(cuda, lib, fft_fused, shape, r_split):
    """pmgb_mesh_forces_f32 on the potential pipeline (one inverse transform
    of the potential, then the order-1 gradient as its real-space stencil:
    the tiled kernel that prefetches the next plane where nx, ny, nz are
    multiples of 32, 8 and 32, one thread per cell otherwise) against the
    oracle's three spectral force meshes of the same density in float64."""
    from jaxpm_gb300 import _lib
    rng = np.random.default_rng(8)
    rho = rng.lognormal(0.0, 0.6, shape).astype(np.float32)
    nx, ny, nz = shape
    mesh = torch.as_tensor(rho).to(cuda)
    out = torch.empty((3,) + shape, device=cuda)
    wsb = lib.pmgb_mesh_forces_workspace_size(nx, ny, nz)
    ws = torch.empty(wsb, dtype=torch.uint8, device=cuda)
    _lib.call("pmgb_mesh_forces_f32", _lib.ptr(mesh), _lib.ptr(out), nx, ny, nz, r_split,
              _lib.ptr(ws), wsb, _lib.stream())
    ref = fourier.force_mesh(fourier.fft3d(rho.astype(np.float64)), r_split, dtype=np.float64)
    got = out.cpu().numpy()
    for c in range(3):
        assert rel_l2(got[c], ref[c]) < 1e-5, (c, rel_l2(got[c], ref[c]))


@pytest.mark.parametrize("shape", [(64, 64, 64), (16, 64, 32), (32, 128, 256)])
def test_mesh_forces_vjp_is_the_adjoint(cuda, lib, shape):
    """pmgb_mesh_forces_vjp_f32 (the stencil's transpose folding the three
    cotangent meshes into the potential's, then the potential transform's
    adjoint) is the transpose of pmgb_mesh_forces_f32:
    <forces(m), g> = <m, vjp(g)> for random m and g."""
    from jaxpm_gb300 import _lib
    rng = np.random.default_rng(9)
    nx, ny, nz = shape
    m = torch.as_tensor(rng.standard_normal(shape).astype(np.float32)).to(cuda)
    g = torch.as_tensor(rng.standard_normal((3,) + shape).astype(np.float32)).to(cuda)
    wsb = lib.pmgb_mesh_forces_workspace_size(nx, ny, nz)
    ws = torch.empty(wsb, dtype=torch.uint8, device=cuda)
    f = torch.empty((3,) + shape, device=cuda)
    gm = torch.empty(shape, device=cuda)
    _lib.call("pmgb_mesh_forces_f32", _lib.ptr(m), _lib.ptr(f), nx, ny, nz, 1.0, _lib.ptr(ws),
              wsb, _lib.stream())
    _lib.call("pmgb_mesh_forces_vjp_f32", _lib.ptr(g), _lib.ptr(gm), nx, ny, nz, 1.0,
              _lib.ptr(ws), wsb, _lib.stream())
    lhs = float((f.double() * g.double()).sum())
    rhs = float((m.double() * gm.double()).sum())
    assert abs(lhs - rhs) <= 1e-4 * (abs(lhs) + abs(rhs)), (lhs, rhs)
