"""CPU restatement of OCC's seminumerical (COSX) exchange -- TEST
INFRASTRUCTURE ONLY: imported by tests/, never by the product.

Restates SemiNumericalExchange's ESP path (src/qm/seminumerical_exchange.cpp):
  :233-250    the grid's partitioned atom grids, the numerical overlap
              S_num = sum_g w_g phi(g) phi(g)^T (:334-372) and the overlap
              projector Q = S_num^-1 S (an LDL^T solve there, a dense solve
              here)
  :517-529    restricted: D2q = Q (2 mo.D), K = 0.25 (K' + K'^T)
  :616-648    unrestricted (mo.D 2 nbf x nbf, alpha block above beta): per
              spin D2q_s = Q (2 D_s), K_s = 0.5 (K'_s + K'_s^T)
  :714-855    the sweep: per atom grid, batches of 128 consecutive points;
              a batch is skipped when max phi < precision; F = (w phi) D2q;
              for every shell pair p >= q whose D2q blocks reach 1e-6,
              V_g(mu, nu) = int phi_mu phi_nu / |r - g| (the ESP integrals of
              the pair at each point), G[:, nu] -= F[:, mu] V and, for
              p != q, G[:, mu] -= F[:, nu] V^T; K' -= phi^T G
with the grid of GridSettings::for_sgx (src/numint/grid_settings.cpp:59-68):
n angular points on every shell, LMG radial precision 1e-5, no pruning, no
reduced H / He grid.  The two screens of the sweep are restated: the shell
pairs are the integral engine's significant ones (a shared origin, or an
overlap block of Frobenius norm >= 1e-12; include/occ/qm/integral_engine.h:
250-275, seminumerical_exchange.cpp:279-318), and a pair is skipped for a
batch when |P - c| - extent >= r + 1 Bohr, with c, r the batch's centroid
and bounding radius and P, extent = sqrt(-ln(1e-12) / p) from the pair's
first most diffuse primitive pair (src/ints/esp.cpp:84-96,
seminumerical_exchange.cpp:771-799).

The ESP integrals are McMurchie-Davidson (Hermite expansion of the Gaussian
product, Hermite Coulomb integrals R_tuv over the Boys function; Helgaker,
Jorgensen, Olsen, Molecular Electronic-Structure Theory, ch. 9), vectorised
over the batch's points.  AOs are contracted Cartesian Gaussians in CCA order
scaled as the collocation scales them (common_fac), pure shells through
the real solid-harmonic transform (m = -l..l; p as (y, z, x)).
"""
import math

import numpy as np
from scipy.special import gamma as _gamma, gammainc

def common_fac(l, pure):
    """src/gto/gto.cpp:7-16."""
    if l == 0:
        return 0.28209479177387814
    if l == 1:
        return 0.4886025119029199
    return math.sqrt((2 * l + 1) / (4 * math.pi)) if pure else 1.0


def boys(nmax, T):
    """F_n(T) for n = 0..nmax, T an array: (nmax + 1, len(T))."""
    T = np.asarray(T, dtype=np.float64)
    out = np.empty((nmax + 1,) + T.shape)
    small = T < 1e-10
    Ts = np.where(small, 1.0, T)
    for n in range(nmax + 1):
        a = n + 0.5
        big = _gamma(a) * gammainc(a, Ts) / (2.0 * Ts ** a)
        ser = 1.0 / (2 * n + 1) - T / (2 * n + 3) + T * T / (2.0 * (2 * n + 5))
        out[n] = np.where(small, ser, big)
    return out


def cart_components(l):
    """(a, b, c) of a shell's Cartesian functions in CCA order."""
    return [(a, b, l - a - b) for a in range(l, -1, -1) for b in range(l - a, -1, -1)]


def spherical_transform(l):
    """Real solid harmonics m = -l..l as combinations of the CCA-ordered
    Cartesian monomials (Helgaker, Jorgensen, Olsen, Molecular
    Electronic-Structure Theory, eqs. 6.4.47-6.4.50): T (2l + 1, ncart)."""
    comps = cart_components(l)
    where = {c: i for i, c in enumerate(comps)}
    T = np.zeros((2 * l + 1, len(comps)))
    f = math.factorial
    for m in range(-l, l + 1):
        am = abs(m)
        N = 1.0 / (2.0 ** am * f(l)) * math.sqrt(2.0 * f(l + am) * f(l - am) /
                                                  (2.0 if m == 0 else 1.0))
        v2_lo = 1 if m < 0 else 0
        v2_hi = 2 * ((am - 1) // 2) + 1 if m < 0 else 2 * (am // 2)
        for t in range((l - am) // 2 + 1):
            for u in range(t + 1):
                for v2 in range(v2_lo, v2_hi + 1, 2):
                    sgn = -1.0 if (t + (v2 - v2_lo) // 2) % 2 else 1.0
                    C = sgn * 0.25 ** t * math.comb(l, t) * math.comb(l - t, am + t) * \
                        math.comb(t, u) * math.comb(am, v2)
                    ex, ey, ez = 2 * t + am - 2 * u - v2, 2 * u + v2, l - 2 * t - am
                    if min(ex, ey, ez) < 0:
                        continue
                    T[m + l, where[(ex, ey, ez)]] += N * C
    return T


class Shell:
    """A contracted shell: Cartesian components in CCA order, the transform
    to its functions (identity for Cartesian shells) and common_fac."""

    def __init__(self, l, origin, exps, coefs, pure):
        self.l = l
        self.A = np.asarray(origin, dtype=np.float64)
        self.exps = np.asarray(exps, dtype=np.float64)
        self.coefs = np.asarray(coefs, dtype=np.float64)
        self.comps = cart_components(l)
        self.T = spherical_transform(l) if pure else np.eye(len(self.comps))
        self.fac = common_fac(l, pure)

    def size(self):
        return self.T.shape[0]


def shells_of(basis):
    return [Shell(s.l, s.origin, s.exponents, s.coefficients, basis.pure) for s in basis.shells]


def ao_values(shells, P):
    """phi (npts, nbf)."""
    P = np.asarray(P, dtype=np.float64)
    cols = []
    for sh in shells:
        d = P - sh.A
        r2 = np.einsum("ij,ij->i", d, d)
        R = np.zeros(len(P))
        for a, c in zip(sh.exps, sh.coefs):
            R += c * np.exp(-a * r2)
        cart = np.stack([d[:, 0] ** i * d[:, 1] ** j * d[:, 2] ** k * R
                         for (i, j, k) in sh.comps], axis=1)
        cols.append(sh.fac * cart @ sh.T.T)
    return np.concatenate(cols, axis=1)


def hermite_E(i, j, a, b, Qx):
    """E^{ij}_t, t = 0..i+j, of the product of x^i e^{-a x^2} and
    x^j e^{-b x^2} centred Qx apart."""
    p = a + b
    q = a * b / p
    E = {}

    def e(i, j, t):
        if t < 0 or t > i + j:
            return 0.0
        key = (i, j, t)
        if key in E:
            return E[key]
        if i == 0 and j == 0:
            v = math.exp(-q * Qx * Qx) if t == 0 else 0.0
        elif j == 0:
            v = e(i - 1, j, t - 1) / (2 * p) - q * Qx / a * e(i - 1, j, t) + (t + 1) * e(i - 1, j, t + 1)
        else:
            v = e(i, j - 1, t - 1) / (2 * p) + q * Qx / b * e(i, j - 1, t) + (t + 1) * e(i, j - 1, t + 1)
        E[key] = v
        return v

    return [e(i, j, t) for t in range(i + j + 1)]


def hermite_R(L, p, PC):
    """R_tuv (t + u + v <= L) for points: dict (t, u, v) -> array."""
    T = p * np.einsum("ij,ij->i", PC, PC)
    F = boys(L, T)
    cache = {}

    def R(t, u, v, n):
        if t < 0 or u < 0 or v < 0:
            return 0.0
        key = (t, u, v, n)
        if key in cache:
            return cache[key]
        if t == u == v == 0:
            val = (-2.0 * p) ** n * F[n]
        elif t > 0:
            val = (t - 1) * R(t - 2, u, v, n + 1) + PC[:, 0] * R(t - 1, u, v, n + 1)
        elif u > 0:
            val = (u - 1) * R(t, u - 2, v, n + 1) + PC[:, 1] * R(t, u - 1, v, n + 1)
        else:
            val = (v - 1) * R(t, u, v - 2, n + 1) + PC[:, 2] * R(t, u, v - 1, n + 1)
        cache[key] = val
        return val

    return lambda t, u, v: R(t, u, v, 0)


def overlap(shells):
    n = sum(s.size() for s in shells)
    S = np.zeros((n, n))
    o1 = 0
    for s1 in shells:
        o2 = 0
        for s2 in shells:
            Sc = np.zeros((len(s1.comps), len(s2.comps)))
            for i, c1 in enumerate(s1.comps):
                for j, c2 in enumerate(s2.comps):
                    v = 0.0
                    for a, ca in zip(s1.exps, s1.coefs):
                        for b, cb in zip(s2.exps, s2.coefs):
                            p = a + b
                            e = 1.0
                            for k in range(3):
                                e *= hermite_E(c1[k], c2[k], a, b, s1.A[k] - s2.A[k])[0]
                            v += ca * cb * e * (math.pi / p) ** 1.5
                    Sc[i, j] = v * s1.fac * s2.fac
            S[o1:o1 + s1.size(), o2:o2 + s2.size()] = s1.T @ Sc @ s2.T.T
            o2 += s2.size()
        o1 += s1.size()
    return S


def esp_pair(s1, s2, C):
    """V[g, i, j] = int phi_i phi_j / |r - C_g| for the functions of two shells."""
    C = np.asarray(C, dtype=np.float64)
    V = np.zeros((len(C), len(s1.comps), len(s2.comps)))
    for a, ca in zip(s1.exps, s1.coefs):
        for b, cb in zip(s2.exps, s2.coefs):
            p = a + b
            P = (a * s1.A + b * s2.A) / p
            R = hermite_R(s1.l + s2.l, p, P - C)
            pref = ca * cb * 2.0 * math.pi / p * s1.fac * s2.fac
            for i, c1 in enumerate(s1.comps):
                for j, c2 in enumerate(s2.comps):
                    Ex = hermite_E(c1[0], c2[0], a, b, s1.A[0] - s2.A[0])
                    Ey = hermite_E(c1[1], c2[1], a, b, s1.A[1] - s2.A[1])
                    Ez = hermite_E(c1[2], c2[2], a, b, s1.A[2] - s2.A[2])
                    acc = 0.0
                    for t, ex in enumerate(Ex):
                        for u, ey in enumerate(Ey):
                            for v, ez in enumerate(Ez):
                                acc = acc + ex * ey * ez * R(t, u, v)
                    V[:, i, j] += pref * acc
    return np.einsum("fi,gij,hj->gfh", s1.T, V, s2.T)


def sgx_grid(basis, angular=110):
    """The partitioned atom grids of GridSettings::for_sgx(angular): points,
    weights and each atom's point count (oracle restatement of the grid)."""
    import grid_oracle as go
    Z, R = go.basis_atoms(basis)
    s = go.Settings(max_angular=angular, min_angular=angular, radial_precision=1e-5,
                    reduced_first_row=False, pruning="none")
    return go.molecular_grid(Z, R, go.basis_shells(basis), s, atom_counts=True)


def pair_geometry(s1, s2):
    """Centre and extent of a shell pair: its first primitive pair (s1's
    primitives outer, s2's inner) of smallest exponent sum p, and
    sqrt(-ln(1e-12) / p)."""
    pmin, P = None, None
    for a in s1.exps:
        for b in s2.exps:
            p = a + b
            if pmin is None or p < pmin:
                pmin, P = p, (a * s1.A + b * s2.A) / p
    return P, math.sqrt(27.631021115928547 / pmin)


def significant_pairs(shells, S, threshold=1e-12):
    """(p, q), p >= q, of a shared origin or overlap block norm >= threshold."""
    first = np.cumsum([0] + [s.size() for s in shells])
    out = []
    for p in range(len(shells)):
        for q in range(p + 1):
            if np.array_equal(shells[p].A, shells[q].A) or \
                    np.linalg.norm(S[first[p]:first[p + 1], first[q]:first[q + 1]]) >= threshold:
                out.append((p, q))
    return out


def cosx_exchange(basis, D, angular=110, precision=np.finfo(np.float64).eps,
                  density_threshold=1e-6, block=128, margin=1.0, grid=None):
    """K (nbf x nbf) of mo.D = D, restricted, ESP path.  grid: (points,
    weights, atom block sizes) instead of for_sgx(angular)."""
    shells = shells_of(basis)
    P, W, counts = grid if grid is not None else sgx_grid(basis, angular)
    phi = ao_values(shells, P)
    Snum = phi.T @ (phi * W[:, None])
    S = overlap(shells)
    Q = np.linalg.solve(Snum, S)
    D2q = Q @ (2.0 * np.asarray(D))
    first = np.cumsum([0] + [s.size() for s in shells])
    nbf = first[-1]
    pairs = significant_pairs(shells, S)
    geo = {pq: pair_geometry(shells[pq[0]], shells[pq[1]]) for pq in pairs}
    K = np.zeros((nbf, nbf))
    off = 0
    for cnt in counts:
        for b0 in range(0, cnt, block):
            idx = slice(off + b0, off + min(cnt, b0 + block))
            ph, w, pts = phi[idx], W[idx], P[idx]
            centre = pts.mean(axis=0)
            radius = np.sqrt(((pts - centre) ** 2).sum(axis=1)).max()
            if ph.max() < precision:
                continue
            F = (ph * w[:, None]) @ D2q
            G = np.zeros_like(F)
            for p, q in pairs:
                Pc, ext = geo[(p, q)]
                if np.linalg.norm(Pc - centre) - ext >= radius + margin:
                    continue
                bp = slice(first[p], first[p + 1])
                bq = slice(first[q], first[q + 1])
                mD = np.abs(D2q[bp, bq]).max()
                if p != q:
                    mD = max(mD, np.abs(D2q[bq, bp]).max())
                if mD < density_threshold:
                    continue
                V = esp_pair(shells[p], shells[q], pts)
                G[:, bq] -= np.einsum("gi,gij->gj", F[:, bp], V)
                if p != q:
                    G[:, bp] -= np.einsum("gj,gij->gi", F[:, bq], V)
            K -= ph.T @ G
        off += cnt
    return 0.25 * (K + K.T)


def cosx_exchange_unrestricted(basis, D, **kw):
    """K (2 nbf x nbf) of an unrestricted mo.D (alpha block above beta):
    per spin 0.5 (K'_s + K'_s^T) of Q (2 D_s), twice the restricted
    expression's 0.25 for the same block (seminumerical_exchange.cpp:616-648)."""
    D = np.asarray(D)
    nbf = D.shape[1]
    return np.vstack([2.0 * cosx_exchange(basis, D[:nbf], **kw),
                      2.0 * cosx_exchange(basis, D[nbf:], **kw)])
