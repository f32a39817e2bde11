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


def _pair_list(pairs):
    s1 = np.floor((np.sqrt(8.0 * pairs + 1) - 1) / 2).astype(np.int64)
    s1 -= (s1 * (s1 + 1) // 2 > pairs)
    s1 += ((s1 + 1) * (s1 + 2) // 2 <= pairs)
    return np.stack([s1, pairs - s1 * (s1 + 1) // 2], 1)


@pytest.mark.parametrize("mode", [0, 1])
def test_noalloc_at_the_size_limit_vs_oracle(setup, oracle_mod, mode):
    # (H2O)32 cc-pVDZ: nbf = 768 = LGX_NOALLOC_MAX_NBF, so the accumulators
    # fill the array to its last element.  The whole screened pass against
    # lgx_jk_device, and a pass restricted to a pair subset that includes the
    # basis's last shell pair against the oracle's J/K over the same quartets.
    torch, lg, _, _ = setup
    import bench
    atoms = lg.water_cluster(4, 4, 2, spacing=3.0, jitter=0.2, seed=2024)
    bs = lg.BasisSet("cc-pVDZ", atoms)
    assert bs.nbf == lg._lgx.LGX_NOALLOC_MAX_NBF
    D = lg.random_density(bs.nbf, 5 * 32, seed=2025)
    ctx = lg.Context(0)
    ctx.set_basis(bs)
    dD = torch.tensor(D, device="cuda")
    dJ, dK = torch.empty_like(dD), torch.empty_like(dD)
    ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), 1e-12, mode, 1e-4)
    Jref, Kref = dJ.cpu().numpy(), dK.cpu().numpy()
    for _ in range(2):
        dJ.fill_(5.0)
        dK.fill_(5.0)
        ctx.jk_device_noalloc(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), 1e-12, mode, 1e-4)
        torch.cuda.synchronize()
        assert np.max(np.abs(dJ.cpu().numpy() - Jref)) < TOL
        assert np.max(np.abs(dK.cpu().numpy() - Kref)) < TOL
    ob = oracle_mod.OracleBasis.from_basis(bs)
    K = oracle_mod.schwarz(ob)
    ns = len(bs)
    last = ns * (ns + 1) // 2 - 1
    pairs = np.union1d(bench.sample_pairs(ob, K, 1e-12, 1500, 3), [last, last - 1])
    acc = oracle_mod.JKAccumulator(ob.nbf)
    acc.add_pairs(ob, D, K, 1e-12, pairs, ket_subset=True)
    Jo, Ko = acc.reduce()
    acc.close()
    assert np.abs(Jo[-1, :]).max() > 0  # the last function's row is touched
    ctx.set_pair_subset(_pair_list(pairs))
    ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), 1e-12, mode, 1e-4)
    for _ in range(2):
        dJ.fill_(5.0)
        dK.fill_(5.0)
        ctx.jk_device_noalloc(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), 1e-12, mode, 1e-4)
        torch.cuda.synchronize()
        J, Kx = dJ.cpu().numpy(), dK.cpu().numpy()
        if mode == 0:
            assert np.max(np.abs(J - Jo)) < 1e-10 and np.max(np.abs(Kx - Ko)) < 1e-10
        else:
            EJ, EK = lg.jk_energies(D, J, Kx)
            EJo, EKo = lg.jk_energies(D, Jo, Ko)
            assert abs(EJ - EJo) < 1e-8 and abs(EK - EKo) < 1e-8
            assert np.max(np.abs(J - Jo)) < 1e-6 and np.max(np.abs(Kx - Ko)) < 1e-6
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_noalloc_tz_after_branched_pass(setup, mode):
    # (H2O)12 cc-pVTZ (nbf = 696): the f-shell classes run on the program
    # kernel with per-warp slot scratch in global memory, which the prepared
    # (branched) pass grows per branch; the no-allocation pass runs every
    # launch on one stream with the largest of those buffers
    torch, lg, _, _ = setup
    atoms = lg.water_cluster(3, 2, 2, spacing=3.0, jitter=0.2, seed=8)
    bs = lg.BasisSet("cc-pVTZ", atoms)
    assert bs.nbf == 696
    D = lg.random_density(bs.nbf, 60, seed=9)
    ctx = lg.Context(0)
    ctx.set_basis(bs)
    dD = torch.tensor(D, device="cuda")
    dJ, dK = torch.empty_like(dD), torch.empty_like(dD)
    ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), 1e-12, mode, 1e-4)
    kinds = {r["kernel"] for r in ctx.last_pass_launches()}
    assert any(k != "register" for k in kinds), kinds
    Jref, Kref = dJ.cpu().numpy(), dK.cpu().numpy()
    for _ in range(2):
        dJ.fill_(-1.0)
        dK.fill_(-1.0)
        ctx.jk_device_noalloc(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), 1e-12, mode, 1e-4)
        torch.cuda.synchronize()
        assert np.max(np.abs(dJ.cpu().numpy() - Jref)) < TOL
        assert np.max(np.abs(dK.cpu().numpy() - Kref)) < TOL
    ctx.close()
