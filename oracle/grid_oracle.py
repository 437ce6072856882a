"""CPU restatement of OCC's molecular integration grid -- TEST INFRASTRUCTURE
ONLY: imported by tests/, never by the product (occ_gb300/ does not import
it).  It is an independent check of the library's grid (the LMG radial grid,
NWChem angular pruning, Lebedev rules and the Becke partition with the
Treutler-Ahlrichs radius adjustment), written in numpy from the reference
sources:

  src/numint/grid_utils.cpp:16-41    Lebedev levels, Bragg radii
  src/numint/grid_utils.cpp:99-107   becke_partition (three iterations)
  src/numint/grid_utils.cpp:125-200  Treutler-Ahlrichs adjustment and the
                                     pairwise cell functions
  src/numint/grid_utils.cpp:234-274  prune_nwchem_scheme
  src/numint/grid_utils.cpp:396-514  lmg_inner / lmg_outer / lmg_h and
                                     generate_lmg_radial_grid
  src/numint/grid_utils.cpp:576-758  generate_atom_grid (LMG + NWChem path)
  src/numint/molecular_grid.cpp:46-82, 142-256
                                     settings checks, per-atom exponent
                                     ranges, per-element atom grids and the
                                     normalised partition

The Lebedev rules are the reference's own table (src/numint/lebedev.cpp),
read from tests/golden/lebedev_ref.npz, which tests/golden/make_golden.py
writes from that source compiled unmodified; the library generates its rules
separately.  The LMG searches keep C's arithmetic where the reference relies
on it: the exponent of an angular momentum that an atom's basis lacks is
DBL_MAX, for which the outer-radius walk meets inf * 0 = NaN and ends near
zero (std::max / std::min then keep the other operand).

Beyond the reference, `refined_grid` replaces the Lebedev rule by a product
rule (Gauss-Legendre in cos(theta) x uniform in phi, exact for spherical
harmonics up to degree 2 n_theta - 1) and tightens the radial precision, so
that integrals can be converged far past the default grid.
"""
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(os.path.dirname(HERE), "tests", "golden", "lebedev_ref.npz")

# src/numint/grid_utils.cpp:16-19
LEVELS = [1, 6, 14, 26, 38, 50, 74, 86, 110, 146, 170, 194, 230, 266, 302, 350, 434, 590, 770,
          974, 1202, 1454, 1730, 2030, 2354, 2702, 3074, 3470, 3890, 4334, 4802, 5294, 5810]
# src/numint/grid_utils.cpp:23-28, H..Ar (Angstrom)
BRAGG = [0.35, 1.40, 1.45, 1.05, 0.85, 0.70, 0.65, 0.60, 0.50, 1.50, 1.80, 1.50, 1.25, 1.10,
         1.00, 1.00, 1.00, 1.80]
ANGSTROM_TO_BOHR = 1.0 / 0.52917721067  # include/occ/core/units.h
DBL_MAX = np.finfo(np.float64).max
FLT_MAX = float(np.finfo(np.float32).max)

_leb = None


def lebedev(n):
    """(n, 4) x, y, z, w of the reference's rule with n points."""
    global _leb
    if _leb is None:
        f = np.load(GOLDEN)
        _leb = {int(k[1:]): f[k] for k in f.files}
    if n not in _leb:
        raise KeyError(f"Lebedev rule {n} is not in the golden table")
    return _leb[n]


def product_rule(nth):
    """Gauss-Legendre (nth) x uniform (2 nth) rule on the unit sphere, weights
    summing to 1 like the Lebedev table's."""
    ct, wt = np.polynomial.legendre.leggauss(nth)
    nph = 2 * nth
    ph = np.arange(nph) * (2.0 * np.pi / nph)
    st = np.sqrt(1.0 - ct * ct)
    x = np.outer(st, np.cos(ph)).ravel()
    y = np.outer(st, np.sin(ph)).ravel()
    z = np.repeat(ct, nph)
    w = np.outer(wt, np.full(nph, 1.0 / nph)).ravel() * 0.5
    return np.stack([x, y, z, w], axis=1)


def level_at_or_above(n):
    for m in LEVELS:
        if m >= n:
            return m
    raise ValueError("Requested number of angular points exceeds 5810")


def level_below(n):
    if n <= LEVELS[0]:
        return LEVELS[0]
    for m in reversed(LEVELS):
        if m < n:
            return m
    return LEVELS[0]


def bragg_radius(Z):
    return BRAGG[Z - 1] * ANGSTROM_TO_BOHR


def _cmax(a, b):  # std::max(a, b): (a < b) ? b : a
    return b if a < b else a


def _cmin(a, b):  # std::min(a, b): (b < a) ? b : a
    return b if b < a else a


def lmg_inner(max_error, alpha_inner):
    """TCA 106, 178 (2001) eq. 25 (grid_utils.cpp:396-405)."""
    m, d = 0, 1.9
    r = d - math.log(1.0 / max_error)
    r = r * 2.0 / (m + 3.0)
    r = math.exp(r) / alpha_inner
    return math.sqrt(r)


def lmg_outer(max_error, alpha_outer, l, guess):
    """Eq. 19, the reference's walk with step division by 10 on each sign
    change (grid_utils.cpp:407-441), in IEEE arithmetic."""
    m = 2 * l
    r = np.float64(guess)
    r_old = np.float64(1.0e50)
    step = np.float64(0.5)
    f = np.float64(1.0e50)
    sign = 1.0 if f > max_error else -1.0
    a_out = np.float64(alpha_outer)
    with np.errstate(over="ignore", invalid="ignore"):
        while abs(r_old - r) > 1e-14:
            c = math.gamma((m + 3.0) / 2.0)
            a = np.power(a_out * r * r, (m + 1.0) / 2.0)
            e = np.exp(-a_out * r * r)
            f = c * a * e
            sign_old = sign
            sign = 1.0 if f > max_error else -1.0
            if r < 0.0:
                sign = 1.0
            if sign != sign_old:
                step *= 0.1
            r_old = r
            r = r + sign * step
    return float(r)


def lmg_h(max_error, l, guess):
    """Eqs. 17-18 (grid_utils.cpp:443-477)."""
    m = 2 * l
    h = np.float64(guess)
    h_old = np.float64(1.0e50)
    step = np.float64(0.1) * guess
    f = 1.0e50
    sign = -1.0 if f > max_error else 1.0
    pi = math.pi
    with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
        while abs(h_old - h) > 1e-14:
            c0 = 4.0 * math.sqrt(2.0) * pi
            cm = math.gamma(3.0 / 2.0) / math.gamma((m + 3.0) / 2.0)
            p0 = 1.0 / h
            e0 = np.exp(-pi * pi / (2.0 * h))
            pm = np.power(pi / h, m / 2.0)
            rd0 = c0 * p0 * e0
            f = cm * pm * rd0
            sign_old = sign
            sign = -1.0 if f > max_error else 1.0
            if h < 0.0:
                sign = 1.0
            if sign != sign_old:
                step *= 0.1
            h_old = h
            h = h + sign * step
    return float(h)


def lmg_radial(Z, precision, alpha_max, l_max, alpha_min):
    """generate_lmg_radial_grid (grid_utils.cpp:479-514): points, weights
    (r^2 included, 4 pi not yet)."""
    r_inner = lmg_inner(precision, 2 * alpha_max)
    h = FLT_MAX
    r_outer = 0.0
    br = bragg_radius(Z)
    for i in range(l_max + 1):
        if alpha_min[i] > 0.0:
            r_outer = _cmax(r_outer, lmg_outer(precision, alpha_min[i], i, 4.0 * br))
            h = _cmin(h, lmg_h(precision, i, 0.1 * (r_outer - r_inner)))
    c = r_inner / (math.exp(h) - 1.0)
    n = int(math.log(1.0 + (r_outer / c)) / h)
    i = np.arange(1, n + 1, dtype=np.float64)
    r = c * (np.exp(i * h) - 1.0)
    w = (r + c) * h * r * r
    return r, w


def prune_nwchem(Z, max_angular, radii):
    """prune_nwchem_scheme (grid_utils.cpp:234-274): Lebedev order per shell."""
    if max_angular < 50:
        return np.full(len(radii), max_angular, dtype=int)
    if max_angular == 50:
        lev = [5, 6, 6, 6, 5]
    else:
        i = 6
        while i < len(LEVELS) and LEVELS[i] != max_angular:
            i += 1
        lev = [5, 6, i - 1, i, i - 1]
    alphas = [0.1, 0.4, 0.8, 2.5]
    if Z <= 2:
        alphas = [0.25, 0.5, 1.0, 4.5]
    elif Z <= 10:
        alphas = [0.16666667, 0.5, 0.9, 3.5]
    radius = bragg_radius(Z)
    out = []
    for r in radii:
        scale = r / radius
        place = next((k for k, a in enumerate(alphas) if a > scale), 4)
        out.append(LEVELS[lev[place]])
    return np.array(out, dtype=int)


class Settings:
    """occ::numint::GridSettings (include/occ/numint/grid_settings.h:81-95)."""

    def __init__(self, max_angular=302, min_angular=110, radial_precision=1e-12,
                 reduced_first_row=True, treutler_ahlrichs=True, pruning="nwchem"):
        self.max_angular = max_angular
        self.min_angular = min_angular
        self.radial_precision = radial_precision
        self.reduced_first_row = reduced_first_row
        self.treutler_ahlrichs = treutler_ahlrichs
        self.pruning = pruning


def atom_grid(Z, s, alpha_max, l_max, alpha_min, product_theta=0):
    """generate_atom_grid, LMG radial method (grid_utils.cpp:576-758):
    (points relative to the nucleus (n, 3), weights (n,)).  With
    product_theta > 0 every shell uses product_rule(product_theta) instead
    of a Lebedev rule (refinement beyond the reference)."""
    if alpha_max <= 0.0 or l_max <= 0 or len(alpha_min) == 0:
        r, wr = lmg_radial(Z, s.radial_precision, 20.0, 3, [0.1] * 4)
    else:
        r, wr = lmg_radial(Z, s.radial_precision, alpha_max, l_max, alpha_min)
    wr = wr * (4.0 * math.pi)
    max_ang = s.max_angular
    if s.reduced_first_row and Z < 3:
        max_ang = level_below(max_ang)
    if s.pruning == "nwchem":
        nang = prune_nwchem(Z, max_ang, r)
    else:
        nang = np.full(len(r), max_ang, dtype=int)
    pts, wts = [], []
    for i in range(len(r)):
        rule = product_rule(product_theta) if product_theta else lebedev(level_at_or_above(nang[i]))
        pts.append(rule[:, :3] * r[i])
        wts.append(rule[:, 3] * wr[i])
    return np.concatenate(pts), np.concatenate(wts)


def becke_cell_weights(P, R, radii, treutler_ahlrichs=True):
    """calculate_atomic_grid_weights_impl (grid_utils.cpp:149-200) with the
    Becke partition: (npts, natom) unnormalised cell functions."""
    natom = len(R)
    d = np.empty((len(P), natom))
    for a in range(natom):
        d[:, a] = np.sqrt(((P - R[a]) ** 2).sum(axis=1))
    W = np.ones((len(P), natom))
    for i in range(natom):
        for j in range(i):
            Rij = math.sqrt(float(((R[i] - R[j]) ** 2).sum()))
            w = (d[:, i] - d[:, j]) / Rij
            ri, rj = radii[i], radii[j]
            if abs(ri - rj) > 1e-14:
                xi = math.sqrt(ri / rj) if treutler_ahlrichs else ri / rj
                u = (xi - 1) / (xi + 1)
                a = u / (u * u - 1.0)
                w = w + a * (1 - w * w)
            for _ in range(3):
                w = (3 - w * w) * w * 0.5
            zero = np.abs(1.0 - w) < 1e-14
            W[:, i] = np.where(zero, 0.0, W[:, i] * 0.5 * (1.0 - w))
            W[:, j] = np.where(zero, W[:, j], W[:, j] * 0.5 * (1.0 + w))
    return W


def exponent_ranges(shells, natom):
    """MolecularGrid::initialize_from_basis (molecular_grid.cpp:183-225):
    per atom alpha_max and alpha_min[l] for l = 0..basis l_max (DBL_MAX where
    the atom has no shell of that l); l_max is the whole basis' for every
    atom.  shells: iterable of (l, atom, exponents)."""
    lmax = max(l for l, _, _ in shells)
    amax = np.zeros(natom)
    amin = np.full((natom, lmax + 1), DBL_MAX)
    for l, a, ex in shells:
        amin[a, l] = min(amin[a, l], float(np.min(ex)))
        amax[a] = max(amax[a], float(np.max(ex)))
    return lmax, amax, amin


def molecular_grid(Z, R, shells, s=None, product_theta=0, chunk=50000, atom_counts=False):
    """Points (n, 3) and weights (n,) in the reference's order (atom blocks,
    radial shells, angular points), Bohr.  Z: atomic numbers, R: (natom, 3)
    Bohr, shells: (l, atom, exponents) per shell.  atom_counts: also return
    the number of points of each atom's block."""
    s = s or Settings()
    # ensure_settings (molecular_grid.cpp:142-181)
    if s.max_angular < s.min_angular:
        s.max_angular = s.min_angular + 1
    s.max_angular = level_at_or_above(s.max_angular)
    s.min_angular = level_at_or_above(s.min_angular)
    Z = [int(z) for z in Z]
    R = np.asarray(R, dtype=np.float64).reshape(-1, 3)
    natom = len(Z)
    lmax, amax, amin = exponent_ranges(shells, natom)
    egrid = {}
    for z in sorted(set(Z)):
        first = Z.index(z)
        egrid[z] = atom_grid(z, s, amax[first], lmax, amin[first], product_theta)
    radii = np.array([bragg_radius(z) for z in Z])
    Ps, Ws = [], []
    for a in range(natom):
        p0, w0 = egrid[Z[a]]
        P = p0 + R[a]
        w = np.empty(len(P))
        for c0 in range(0, len(P), chunk):
            cw = becke_cell_weights(P[c0:c0 + chunk], R, radii, s.treutler_ahlrichs)
            w[c0:c0 + chunk] = w0[c0:c0 + chunk] * cw[:, a] / cw.sum(axis=1)
        Ps.append(P)
        Ws.append(w)
    if atom_counts:
        return np.concatenate(Ps), np.concatenate(Ws), [len(w) for w in Ws]
    return np.concatenate(Ps), np.concatenate(Ws)


def becke_radial(n, rm):
    """Becke's radial rule (JCP 88, 2547 (1988)): Gauss-Chebyshev of the second
    kind on x, r = rm (1 + x) / (1 - x); weights include r^2."""
    i = np.arange(1, n + 1, dtype=np.float64)
    x = np.cos(i * np.pi / (n + 1))
    wx = np.pi / (n + 1) * np.sin(i * np.pi / (n + 1)) ** 2 / np.sqrt(1.0 - x * x)
    r = rm * (1.0 + x) / (1.0 - x)
    return r, wx * 2.0 * rm / (1.0 - x) ** 2 * r * r


def refined_grid(Z, R, nrad, ntheta, chunk=50000):
    """A grid for converging integrals far beyond the default one: per atom
    Becke's radial rule with nrad points (rm = the Bragg radius, half of it
    for H) times product_rule(ntheta) on every shell, partitioned like the
    molecular grid (Becke cells with the Treutler-Ahlrichs adjustment).  The
    converged integral does not depend on the partition."""
    Z = [int(z) for z in Z]
    R = np.asarray(R, dtype=np.float64).reshape(-1, 3)
    radii = np.array([bragg_radius(z) for z in Z])
    ang = product_rule(ntheta)
    Ps, Ws = [], []
    for a, z in enumerate(Z):
        r, wr = becke_radial(nrad, bragg_radius(z) * (0.5 if z == 1 else 1.0))
        P = (r[:, None, None] * ang[None, :, :3]).reshape(-1, 3) + R[a]
        w0 = (wr[:, None] * ang[None, :, 3]).ravel() * (4.0 * math.pi)
        w = np.empty(len(P))
        for c0 in range(0, len(P), chunk):
            cw = becke_cell_weights(P[c0:c0 + chunk], R, radii)
            w[c0:c0 + chunk] = w0[c0:c0 + chunk] * cw[:, a] / cw.sum(axis=1)
        Ps.append(P)
        Ws.append(w)
    return np.concatenate(Ps), np.concatenate(Ws)


def basis_shells(basis):
    """(l, atom, exponents) per shell of an occ_gb300.AOBasis."""
    return [(s.l, s.atom, np.asarray(s.exponents, dtype=np.float64)) for s in basis.shells]


def basis_atoms(basis):
    atoms = basis.atoms()
    Z = [a.atomic_number for a in atoms]
    R = np.array([[a.x, a.y, a.z] for a in atoms], dtype=np.float64)
    return Z, R
