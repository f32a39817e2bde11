"""lgx_jk_device_noalloc: the J/K pass for callers that cannot allocate device
memory during the call (its accumulators live in a fixed __device__ array
of the library).  Checked through the C ABI against lgx_jk_device on the
same inputs, on two calls in a row, at the J/K tolerance of the other GPU
tests; plus its size limit and its preparation requirement.  This file is
collected last so a failure here never hides the other tests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-11


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    import libint_gb300 as lg
    atoms = lg.water_cluster(2, 2, 1, spacing=3.0, jitter=0.2, seed=5)
    bs = lg.BasisSet("cc-pVDZ", atoms)
    D = lg.random_density(bs.nbf, 20, seed=6)
    return torch, lg, bs, D


@pytest.mark.parametrize("mode", [0, 1])
def test_noalloc_matches_jk_device_twice(setup, mode):
    torch, lg, bs, D = setup
    ctx = lg.Context(0)
    ctx.set_basis(bs)
    dD = torch.tensor(D, device="cuda")
    dJ = torch.empty_like(dD)
    dK = torch.empty_like(dD)
    ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), 1e-12, mode, 1e-4)
    torch.cuda.synchronize()
    Jref, Kref = dJ.cpu().numpy(), dK.cpu().numpy()
    for _ in range(2):
        dJ.fill_(123.0)
        dK.fill_(-7.0)
        torch.cuda.synchronize()
        ctx.jk_device_noalloc(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), 1e-12, mode, 1e-4)
        torch.cuda.synchronize()
        assert np.max(np.abs(dJ.cpu().numpy() - Jref)) < TOL
        assert np.max(np.abs(dK.cpu().numpy() - Kref)) < TOL
    ctx.close()


def test_noalloc_needs_prepared_state(setup):
    torch, lg, bs, D = setup
    ctx = lg.Context(0)
    ctx.set_basis(bs)
    dD = torch.tensor(D, device="cuda")
    dJ = torch.empty_like(dD)
    dK = torch.empty_like(dD)
    with pytest.raises(lg.LgxError) as e:
        ctx.jk_device_noalloc(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), 1e-12, 0, 1e-4)
    assert e.value.status == lg._lgx.LGX_ERR_INVALID_ARG
    assert "not prepared" in str(e.value)
    ctx.close()


def test_noalloc_rejects_basis_above_limit(setup):
    torch, lg, _, _ = setup
    atoms = lg.water_cluster(4, 4, 1, spacing=3.0, jitter=0.2, seed=5)
    bs = lg.BasisSet("cc-pVDZ", atoms)  # 16 waters x 24 functions = 384
    bs2 = lg.BasisSet("cc-pVTZ", atoms)  # 16 waters x 58 functions = 928
    assert bs.nbf <= lg._lgx.LGX_NOALLOC_MAX_NBF < bs2.nbf
    ctx = lg.Context(0)
    ctx.set_basis(bs2)
    n = bs2.nbf
    dD = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    with pytest.raises(lg.LgxError) as e:
        ctx.jk_device_noalloc(dD.data_ptr(), dD.data_ptr(), dD.data_ptr(), 1e-12, 0, 1e-4)
    assert e.value.status == lg._lgx.LGX_ERR_TOO_LARGE
    assert "LGX_NOALLOC_MAX_NBF" in str(e.value)
    ctx.close()
