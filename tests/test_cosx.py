"""Seminumerical (COSX) exchange, the ESP form of OCC's SemiNumericalExchange
(src/qm/seminumerical_exchange.cpp:233-250, :516-529, :714-855).

CPU: the oracle (oracle/cosx_oracle.py) is pinned against the exact
exchange matrix of the same density from four-centre integrals
(tests/golden/make_hf_density.py), on the reference's own test system
(tests/dft_tests.cpp:322-347, 371-418: water, 6-31G Cartesian, RHF density,
GridSettings::for_sgx(50) and (110)); its analytic overlap against that
file's overlap, its AO values against the collocation oracle, and its grid
against the library's host grid.
GPU: the library's K against the oracle's at 1e-9 (FP64 throughout); the
mixed precision (ESP integrals in FP32) against FP64."""
import os
import sys

import numpy as np
import pytest

import occ_gb300 as og
import oracle
import cosx_oracle as cx
import grid_oracle as go

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_hf_density as hf  # noqa: E402

WATER = [(8, -1.32695761, -0.10593856, 0.01878821),
         (1, -1.93166418, 1.60017351, -0.02171049),
         (1, 0.48664409, 0.07959806, 0.00986248)]
TOL_GPU = 1e-9


def _water(basis="6-31g", pure=False, shift=(0.0, 0.0, 0.0)):
    atoms = [og.Atom(z, x + shift[0], y + shift[1], w + shift[2]) for z, x, y, w in WATER]
    b = og.AOBasis.load(atoms, basis)
    b.set_pure(pure)
    return atoms, b


_CACHE = {}


def _rhf_water_631g():
    """RHF density and exact K of water / 6-31G (Cartesian), as the
    reference's test computes them (SCF, then HartreeFock::compute_JK)."""
    if "rhf" not in _CACHE:
        atoms, b = _water()
        Z = np.array([a.atomic_number for a in atoms], dtype=float)
        xyz = np.array([[a.x, a.y, a.z] for a in atoms])
        enuc = sum(Z[i] * Z[j] / np.linalg.norm(xyz[i] - xyz[j])
                   for i in range(3) for j in range(i))
        aos = hf.ao_list(b)
        S, T, V = hf.one_electron(aos, Z, xyz)
        G = hf.eri(aos)
        _, D, _ = hf.rhf(S, T + V, G, 5, enuc)
        K = np.einsum("ls,mlns->mn", D, G)
        _CACHE["rhf"] = (b, D, K, S)
    return _CACHE["rhf"]


def test_oracle_overlap_and_ao_values_match_independent_forms():
    b, _, _, S = _rhf_water_631g()
    shells = cx.shells_of(b)
    assert np.abs(cx.overlap(shells) - S).max() < 1e-13
    P = np.random.default_rng(0).normal(size=(50, 3))
    col = [oracle.collocation(s.l, b.pure, s.exponents, s.coefficients, s.origin, P,
                              deriv=0)[0].T for s in b.shells]
    assert np.abs(np.concatenate(col, axis=1) - cx.ao_values(shells, P)).max() < 1e-14
    # pure d shells through the solid-harmonic transform
    _, bp = _water("def2-svp", pure=True)
    col = [oracle.collocation(s.l, bp.pure, s.exponents, s.coefficients, s.origin, P,
                              deriv=0)[0].T for s in bp.shells]
    assert np.abs(np.concatenate(col, axis=1) - cx.ao_values(cx.shells_of(bp), P)).max() < 1e-14


def test_oracle_boys_function_limits():
    T = np.array([0.0, 1e-12, 0.5, 7.0, 30.0, 60.0])
    F = cx.boys(4, T)
    assert np.allclose(F[:, 0], 1.0 / (2 * np.arange(5) + 1), rtol=0, atol=1e-15)
    assert abs(F[0, -1] - 0.5 * np.sqrt(np.pi / 60.0)) < 1e-15
    # downward recursion F_{n-1} = (2T F_n + e^-T) / (2n - 1)
    for n in range(1, 5):
        assert np.allclose(F[n - 1], (2 * T * F[n] + np.exp(-T)) / (2 * n - 1), rtol=1e-13)


@pytest.mark.parametrize("angular,bar", [(50, 5e-4), (110, 5e-5)])
def test_oracle_exchange_approaches_exact_exchange(angular, bar):
    """max |K_COSX - K_exact| on water / 6-31G: 3.0e-4 at 50 angular points,
    2.0e-5 at 110 (max |K| 4.9); the reference test prints the same
    difference (tests/dft_tests.cpp:346-347)."""
    b, D, K, _ = _rhf_water_631g()
    Kc = cx.cosx_exchange(b, D, angular=angular)
    assert np.abs(Kc - Kc.T).max() < 1e-14
    err = np.abs(Kc - K).max()
    assert err < bar, err


def test_oracle_unrestricted_approaches_exact_exchange():
    """The unrestricted oracle (seminumerical_exchange.cpp:616-648: per spin
    0.5 (K' + K'^T) of Q (2 D_s), D_s = 0.5 C_s C_s^T as OCC stores it)
    against each spin's exact exchange K_s = (ml|ns) (C_s C_s^T)_ls on water /
    6-31G at for_sgx(50): 1.6e-4 of max |K_s| measured with these random
    orbitals (the restricted RHF test: 6e-5), where a wrong spin factor would
    be off by max |K_s| itself; and a closed shell (D_a = D_b = D / 2) giving
    the restricted K in both blocks."""
    b, D, _, _ = _rhf_water_631g()
    n = b.nbf()
    G = hf.eri(hf.ao_list(b))
    rng = np.random.default_rng(3)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    Ca, Cb = Q[:, :5], Q[:, 1:5]
    Du = np.vstack([0.5 * Ca @ Ca.T, 0.5 * Cb @ Cb.T])
    Ku = cx.cosx_exchange_unrestricted(b, Du, angular=50)
    for Cs, blk in ((Ca, Ku[:n]), (Cb, Ku[n:])):
        Kx = np.einsum("ls,mlns->mn", Cs @ Cs.T, G)
        rel = np.abs(blk - Kx).max() / np.abs(Kx).max()
        assert rel < 2.5e-4, rel
    Kc = cx.cosx_exchange_unrestricted(b, np.vstack([0.5 * D, 0.5 * D]), angular=50)
    Kr = cx.cosx_exchange(b, D, angular=50)
    assert np.abs(Kc[:n] - Kr).max() < 1e-13 and np.abs(Kc[n:] - Kr).max() < 1e-13


def test_oracle_screens_act_on_separated_waters():
    """Two waters 7 Angstrom apart with a density that does not couple them
    (the screen relies on the decay of D): the geometric screen skips far
    pairs in far batches, and what it drops is small."""
    atoms1, _ = _water()
    atoms2, _ = _water(shift=(0.0, 0.0, 7.0))
    b = og.AOBasis.load(atoms1 + atoms2, "sto-3g")
    b.set_pure(False)
    n = b.nbf()
    C = np.random.default_rng(3).normal(size=(n // 2, 5)) * 0.3
    D = np.zeros((n, n))
    D[:n // 2, :n // 2] = C @ C.T
    D[n // 2:, n // 2:] = C @ C.T
    shells = cx.shells_of(b)
    P, W, counts = cx.sgx_grid(b, 26)
    skipped = 0
    pairs = cx.significant_pairs(shells, cx.overlap(shells))
    off = 0
    for cnt in counts:
        for b0 in range(0, cnt, 128):
            pts = P[off + b0:off + min(cnt, b0 + 128)]
            c = pts.mean(axis=0)
            r = np.sqrt(((pts - c) ** 2).sum(axis=1)).max()
            for pq in pairs:
                Pc, ext = cx.pair_geometry(shells[pq[0]], shells[pq[1]])
                skipped += np.linalg.norm(Pc - c) - ext >= r + 1.0
        off += cnt
    assert skipped > 0
    K = cx.cosx_exchange(b, D, grid=(P, W, counts))
    K_all = cx.cosx_exchange(b, D, grid=(P, W, counts), margin=np.inf)
    assert 0.0 < np.abs(K - K_all).max() < 2e-4


def test_oracle_sgx_grid_is_the_library_host_grid():
    _, b = _water()
    P, W, counts = cx.sgx_grid(b, 50)
    gs = og.GridSettings.for_sgx(50)
    Pl, Wl = og.molecular_grid(b, gs)
    assert len(W) == len(Wl) == sum(counts)
    assert np.abs(P - Pl).max() < 1e-12
    assert np.abs(W - Wl).max() < 1e-12 * np.abs(W).max()


def _gpu_case(b, D, grid):
    dft = og.DFT("lda", b)
    sgx = og.SemiNumericalExchange(dft, grid)
    assert sgx.grid_points() == len(og.molecular_grid(b, grid)[1])
    return dft, sgx, sgx.compute_K(D)


@pytest.mark.gpu
@pytest.mark.parametrize("angular", [50, 110])
def test_gpu_cosx_matches_oracle_water_631g(angular):
    b, D, K, _ = _rhf_water_631g()
    _, _, Kg = _gpu_case(b, D, og.GridSettings.for_sgx(angular))
    Ko = cx.cosx_exchange(b, D, angular=angular)
    assert np.abs(Kg - Kg.T).max() < 1e-14
    assert np.abs(Kg - Ko).max() < TOL_GPU, np.abs(Kg - Ko).max()


@pytest.mark.gpu
def test_gpu_cosx_pure_d_two_waters():
    """def2-SVP (pure d shells) on two waters, a random symmetric density."""
    atoms1, _ = _water()
    atoms2, _ = _water(shift=(0.0, 0.0, 5.5))
    b = og.AOBasis.load(atoms1 + atoms2, "def2-svp")
    b.set_pure(True)
    n = b.nbf()
    rng = np.random.default_rng(7)
    C = rng.normal(size=(n, 10)) * 0.3
    D = C @ C.T
    _, sgx, Kg = _gpu_case(b, D, og.GridSettings.for_sgx(50))
    Ko = cx.cosx_exchange(b, D, angular=50)
    assert np.abs(Kg - Ko).max() < TOL_GPU * max(1.0, np.abs(Ko).max())
    # the device entry point writes the same K
    import torch
    dD = torch.tensor(np.asfortranarray(D).ravel(order="F"), device="cuda", dtype=torch.float64)
    dK = torch.empty(n * n, device="cuda", dtype=torch.float64)
    sgx.compute_K_device(dD.data_ptr(), dK.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    Kd = dK.cpu().numpy().reshape(n, n, order="F")
    assert np.abs(Kd - Kg).max() < 1e-13


@pytest.mark.gpu
def test_gpu_cosx_refuses_f_shells_and_bad_grid():
    _, b = _water("def2-tzvp", pure=True)
    dft = og.DFT("lda", b)
    with pytest.raises(og.XCError) as e:
        og.SemiNumericalExchange(dft)
    assert e.value.code == -1
    _, b = _water()
    dft = og.DFT("lda", b)
    with pytest.raises(og.XCError):
        og.SemiNumericalExchange(dft, og.GridSettings(max_angular_points=0))


TOL_K_MIXED = 1e-6  # relative to max |K|: FP32 ESP integrals against FP64 (3e-8 measured)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["water_631g", "two_waters_svp"])
def test_gpu_cosx_mixed_precision(case):
    """The ESP integrals and F in FP32, F and K' formed in double-float FP32
    arithmetic, G and K' summed in FP64: K against the FP64 build, far inside
    COSX's own error against exact exchange (3e-4 of max |K| on water /
    6-31G at for_sgx(50))."""
    if case == "water_631g":
        b, D, _, _ = _rhf_water_631g()
    else:
        atoms1, _ = _water()
        atoms2, _ = _water(shift=(0.0, 0.0, 5.5))
        b = og.AOBasis.load(atoms1 + atoms2, "def2-svp")
        b.set_pure(True)
        C = np.random.default_rng(7).normal(size=(b.nbf(), 10)) * 0.3
        D = C @ C.T
    dft = og.DFT("lda", b)
    sgx = og.SemiNumericalExchange(dft, og.GridSettings.for_sgx(50))
    K64 = sgx.compute_K(D)
    sgx.set_precision(og.MIXED)
    Km = sgx.compute_K(D)
    assert np.abs(Km - Km.T).max() < 1e-14
    rel = np.abs(Km - K64).max() / np.abs(K64).max()
    assert rel <= TOL_K_MIXED, rel
    sgx.set_precision(og.FP64)
    assert np.abs(sgx.compute_K(D) - K64).max() < 1e-13


def _open_shell_density(n, na, nb, seed):
    """An unrestricted mo.D (alpha block above beta, each 0.5 C_s C_s^T) of
    random orbitals, na alpha and nb beta."""
    rng = np.random.default_rng(seed)
    Ca = rng.normal(size=(n, na)) * 0.3
    Cb = rng.normal(size=(n, nb)) * 0.3
    return np.vstack([0.5 * Ca @ Ca.T, 0.5 * Cb @ Cb.T])


@pytest.mark.gpu
def test_gpu_cosx_unrestricted_matches_oracle():
    """compute_K of an unrestricted mo (seminumerical_exchange.cpp:616-648) on
    water / 6-31G: each spin block against the oracle, the host and device
    entry points equal, and a closed shell (D_a = D_b = D / 2) giving the
    restricted K of D in both blocks."""
    _, b = _water()
    n = b.nbf()
    Du = _open_shell_density(n, 5, 4, seed=11)
    dft = og.DFT("lda", b)
    sgx = og.SemiNumericalExchange(dft, og.GridSettings.for_sgx(50))
    Ku = sgx.compute_K(Du)
    assert Ku.shape == (2 * n, n)
    Ko = cx.cosx_exchange_unrestricted(b, Du, angular=50)
    assert np.abs(Ku - Ko).max() < TOL_GPU * max(1.0, np.abs(Ko).max()), np.abs(Ku - Ko).max()
    for s in (slice(0, n), slice(n, 2 * n)):
        assert np.abs(Ku[s] - Ku[s].T).max() < 1e-14
    import torch
    dD = torch.tensor(np.asfortranarray(Du).ravel(order="F"), device="cuda", dtype=torch.float64)
    dK = torch.empty(2 * n * n, device="cuda", dtype=torch.float64)
    sgx.compute_K_device(dD.data_ptr(), dK.data_ptr(), torch.cuda.current_stream().cuda_stream,
                         unrestricted=True)
    torch.cuda.synchronize()
    assert np.abs(dK.cpu().numpy().reshape(2 * n, n, order="F") - Ku).max() < 1e-13
    D = 2.0 * Du[:n]
    Kr = sgx.compute_K(D)
    Kc = sgx.compute_K(np.vstack([0.5 * D, 0.5 * D]))
    assert np.abs(Kc[:n] - Kr).max() < 1e-13 and np.abs(Kc[n:] - Kr).max() < 1e-13


@pytest.mark.gpu
def test_gpu_cosx_unrestricted_mixed_precision():
    """The mixed precision on an unrestricted mo: both blocks within
    TOL_K_MIXED of max |K| of the FP64 build."""
    atoms1, _ = _water()
    atoms2, _ = _water(shift=(0.0, 0.0, 5.5))
    b = og.AOBasis.load(atoms1 + atoms2, "def2-svp")
    b.set_pure(True)
    Du = _open_shell_density(b.nbf(), 10, 9, seed=5)
    dft = og.DFT("lda", b)
    sgx = og.SemiNumericalExchange(dft, og.GridSettings.for_sgx(50))
    K64 = sgx.compute_K(Du)
    sgx.set_precision(og.MIXED)
    Km = sgx.compute_K(Du)
    rel = np.abs(Km - K64).max() / np.abs(K64).max()
    assert rel <= TOL_K_MIXED, rel
