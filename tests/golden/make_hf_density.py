"""Generate water_hf_321g.npz: the converged RHF density of the water molecule
of the reference's isolated XC tests (tests/isolated_xc_tests.cpp:28-56:
O (0, 0, 0), H (0, -0.757, 0.587), H (0, 0.757, 0.587) Angstrom, 3-21G,
set_pure(true), occ::qm::HartreeFock + SCF), so that the E_xc and XC gradient
values those tests assert can be checked here.

The reference obtains the density from libcint integrals, which are not
available here; 3-21G holds only s and p shells, so this script computes the
one- and two-electron integrals itself (McMurchie-Davidson: Hermite expansion
of Gaussian products, Hermite Coulomb integrals over the Boys function; the
textbook scheme of Helgaker, Jorgensen and Olsen, ch. 9) over the AOs exactly
as the collocation evaluates them (common_fac(l) times the normalised
contraction; pure p in OCC's (y, z, x) order), and converges a closed-shell
Roothaan-Hall SCF with DIIS to a commutator norm below 1e-11.  The converged
closed-shell density of the ground state does not depend on the SCF
algorithm.

usage: python tests/golden/make_hf_density.py
"""
import os
import sys
from functools import lru_cache

import numpy as np
from scipy.special import gamma, gammainc

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

import occ_gb300 as og  # noqa: E402

COMMON_FAC = {0: 0.28209479177387814, 1: 0.4886025119029199}  # src/gto/gto.cpp:7-16


def boys(n, T):
    if T < 1e-10:
        return 1.0 / (2 * n + 1) - T / (2 * n + 3) + T * T / (2 * (2 * n + 5))
    return gamma(n + 0.5) * gammainc(n + 0.5, T) / (2.0 * T ** (n + 0.5))


def hermite_E(i, j, a, b, Qx):
    """E^{ij}_t for t = 0..i+j (Gaussian product a at A, b at B, Qx = A - B)."""
    p = a + b
    q = a * b / p

    @lru_cache(maxsize=None)
    def E(i, j, t):
        if t < 0 or t > i + j:
            return 0.0
        if i == 0 and j == 0:
            return np.exp(-q * Qx * Qx) if t == 0 else 0.0
        if j == 0:
            return (E(i - 1, j, t - 1) / (2 * p) - q * Qx / a * E(i - 1, j, t) +
                    (t + 1) * E(i - 1, j, t + 1))
        return (E(i, j - 1, t - 1) / (2 * p) + q * Qx / b * E(i, j - 1, t) +
                (t + 1) * E(i, j - 1, t + 1))

    return [E(i, j, t) for t in range(i + j + 1)]


def hermite_R(L, p, PC):
    """R^0_{tuv} for t + u + v <= L."""
    T = p * float(PC @ PC)
    Fn = [boys(n, T) for n in range(L + 1)]
    cache = {}

    def R(t, u, v, n):
        key = (t, u, v, n)
        if key in cache:
            return cache[key]
        if t < 0 or u < 0 or v < 0:
            return 0.0
        if t == u == v == 0:
            val = (-2.0 * p) ** n * Fn[n]
        elif t > 0:
            val = (t - 1) * R(t - 2, u, v, n + 1) + PC[0] * R(t - 1, u, v, n + 1)
        elif u > 0:
            val = (u - 1) * R(t, u - 2, v, n + 1) + PC[1] * R(t, u - 1, v, n + 1)
        else:
            val = (v - 1) * R(t, u, v - 2, n + 1) + PC[2] * R(t, u, v - 1, n + 1)
        cache[key] = val
        return val

    return lambda t, u, v: R(t, u, v, 0)


class Prim:
    __slots__ = ("c", "a", "A", "lmn")

    def __init__(self, c, a, A, lmn):
        self.c, self.a, self.A, self.lmn = c, a, np.asarray(A, dtype=float), lmn


def ao_list(basis):
    aos = []
    for s in basis.shells:
        if s.l > 1:
            raise SystemExit("this generator handles s and p shells only")
        comps = [(0, 0, 0)] if s.l == 0 else (
            [(0, 1, 0), (0, 0, 1), (1, 0, 0)] if basis.pure else [(1, 0, 0), (0, 1, 0), (0, 0, 1)])
        for lmn in comps:
            aos.append([Prim(COMMON_FAC[s.l] * c, e, s.origin, lmn)
                        for e, c in zip(s.exponents, s.coefficients)])
    return aos


def pair(pa, pb):
    a, b = pa.a, pb.a
    p = a + b
    P = (a * pa.A + b * pb.A) / p
    Es = [hermite_E(pa.lmn[k], pb.lmn[k], a, b, pa.A[k] - pb.A[k]) for k in range(3)]
    return p, P, Es


def one_electron(aos, charges, centres):
    n = len(aos)
    S = np.zeros((n, n))
    T = np.zeros((n, n))
    V = np.zeros((n, n))
    for i in range(n):
        for j in range(i + 1):
            s = t = v = 0.0
            for pa in aos[i]:
                for pb in aos[j]:
                    p, P, Es = pair(pa, pb)
                    cc = pa.c * pb.c
                    ov = [Es[k][0] * np.sqrt(np.pi / p) for k in range(3)]
                    s += cc * ov[0] * ov[1] * ov[2]
                    # kinetic: -1/2 <a| d^2/dx^2 |b> per direction
                    kin = []
                    for k in range(3):
                        lj = pb.lmn[k]
                        b = pb.a

                        def Sk(jj):
                            if jj < 0:
                                return 0.0
                            return hermite_E(pa.lmn[k], jj, pa.a, b, pa.A[k] - pb.A[k])[0] * \
                                np.sqrt(np.pi / p)
                        kin.append(b * (2 * lj + 1) * Sk(lj) - 2 * b * b * Sk(lj + 2) -
                                   0.5 * lj * (lj - 1) * Sk(lj - 2))
                    t += cc * (kin[0] * ov[1] * ov[2] + ov[0] * kin[1] * ov[2] +
                               ov[0] * ov[1] * kin[2])
                    L = sum(pa.lmn) + sum(pb.lmn)
                    for Z, C in zip(charges, centres):
                        R = hermite_R(L, p, P - C)
                        acc = 0.0
                        for tt, ex in enumerate(Es[0]):
                            for uu, ey in enumerate(Es[1]):
                                for vv, ez in enumerate(Es[2]):
                                    acc += ex * ey * ez * R(tt, uu, vv)
                        v -= Z * cc * 2 * np.pi / p * acc
            S[i, j] = S[j, i] = s
            T[i, j] = T[j, i] = t
            V[i, j] = V[j, i] = v
    return S, T, V


def eri(aos):
    n = len(aos)
    prim_pairs = {}
    for i in range(n):
        for j in range(i + 1):
            lst = []
            for pa in aos[i]:
                for pb in aos[j]:
                    p, P, Es = pair(pa, pb)
                    lst.append((pa.c * pb.c, p, P, Es))
            prim_pairs[i, j] = lst
    G = np.zeros((n, n, n, n))
    pairs = sorted(prim_pairs)
    for x, (i, j) in enumerate(pairs):
        for (k, l) in pairs[:x + 1]:
            val = 0.0
            for c1, p, P, E1 in prim_pairs[i, j]:
                for c2, q, Q, E2 in prim_pairs[k, l]:
                    alpha = p * q / (p + q)
                    L = sum(len(e) - 1 for e in E1) + sum(len(e) - 1 for e in E2)
                    R = hermite_R(L, alpha, P - Q)
                    acc = 0.0
                    for t, ex in enumerate(E1[0]):
                        for u, ey in enumerate(E1[1]):
                            for v, ez in enumerate(E1[2]):
                                e1 = ex * ey * ez
                                if e1 == 0.0:
                                    continue
                                for tau, fx in enumerate(E2[0]):
                                    for nu, fy in enumerate(E2[1]):
                                        for phi, fz in enumerate(E2[2]):
                                            sgn = -1.0 if (tau + nu + phi) % 2 else 1.0
                                            acc += e1 * sgn * fx * fy * fz * R(t + tau, u + nu,
                                                                               v + phi)
                    val += c1 * c2 * 2 * np.pi ** 2.5 / (p * q * np.sqrt(p + q)) * acc
            for a, b in ((i, j), (j, i)):
                for c, d in ((k, l), (l, k)):
                    G[a, b, c, d] = G[c, d, a, b] = val
    return G


def rhf(S, H, G, nocc, enuc, tol=1e-11, maxiter=200):
    s, U = np.linalg.eigh(S)
    X = U @ np.diag(s ** -0.5) @ U.T
    F = H.copy()
    errs, focks = [], []
    E_old = 0.0
    for it in range(maxiter):
        e, Cp = np.linalg.eigh(X.T @ F @ X)
        C = X @ Cp
        D = C[:, :nocc] @ C[:, :nocc].T          # OCC's mo.D; P = 2 D
        P = 2 * D
        J = np.einsum("ijkl,kl->ij", G, P)
        K = np.einsum("ikjl,kl->ij", G, P)
        F = H + J - 0.5 * K
        E = 0.5 * np.sum(P * (H + F)) + enuc
        err = F @ P @ S - S @ P @ F
        errs.append(err)
        focks.append(F.copy())
        errs, focks = errs[-8:], focks[-8:]
        if np.max(np.abs(err)) < tol and abs(E - E_old) < 1e-13:
            e, Cp = np.linalg.eigh(X.T @ F @ X)
            C = X @ Cp
            D = C[:, :nocc] @ C[:, :nocc].T
            return E, D, it
        E_old = E
        if len(errs) > 1:  # DIIS extrapolation of F
            m = len(errs)
            B = -np.ones((m + 1, m + 1))
            B[m, m] = 0.0
            for a in range(m):
                for b in range(m):
                    B[a, b] = np.sum(errs[a] * errs[b])
            rhs = np.zeros(m + 1)
            rhs[m] = -1.0
            w = np.linalg.solve(B, rhs)[:m]
            F = sum(wi * Fi for wi, Fi in zip(w, focks))
    raise SystemExit("SCF did not converge")


def main():
    mol = og.Molecule([8, 1, 1], [[0.0, 0.0, 0.0], [0.0, -0.757, 0.587], [0.0, 0.757, 0.587]])
    basis = og.AOBasis.load(mol.atoms(), "3-21g")
    basis.set_pure(True)
    atoms = basis.atoms()
    Z = np.array([a.atomic_number for a in atoms], dtype=float)
    xyz = np.array([[a.x, a.y, a.z] for a in atoms])
    aos = ao_list(basis)
    S, T, V = one_electron(aos, Z, xyz)
    assert np.max(np.abs(np.diag(S) - 1.0)) < 1e-12, np.diag(S)
    G = eri(aos)
    enuc = sum(Z[a] * Z[b] / np.linalg.norm(xyz[a] - xyz[b])
               for a in range(3) for b in range(a))
    E, D, it = rhf(S, T + V, G, 5, enuc)
    print(f"RHF/3-21G water: E = {E:.12f} Ha after {it} iterations, nbf {len(aos)}, "
          f"tr(2DS) = {np.sum(2 * D * S):.12f}")
    np.savez_compressed(os.path.join(HERE, "water_hf_321g.npz"), D=D, hf_energy=np.array(E),
                        S=S, xyz_bohr=xyz, Z=Z)


if __name__ == "__main__":
    main()
