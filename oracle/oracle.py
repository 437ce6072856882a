"""Python access to the CPU oracle (oracle/xc_oracle.cpp) -- TEST
INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py, never by the product.

The oracle restates OCC's restricted XC build on the CPU in FP64
(include/occ/dft/dft.h:192-388).  Its collocation is pinned against the
reference's gau2grid and its PBE exchange against tests/dft_tests.cpp:71-111;
the remaining functionals are restated from their papers (Libxc is not
available here).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_long)
_lib = None

# Libxc ids of the components of OCC's method names (share/methods/dft_methods.json)
METHODS = {
    "lda": [1, 30], "svwn": [1, 30], "lsda": [1, 30], "svwn5": [1, 7],
    "pbe": [101, 130], "blyp": [106, 131], "bpbe": [106, 130],
    "b3lyp": [402], "b3lyp5": [475], "tpss": [202, 231], "vwn5": [7],
    "pbeh": [406], "bhandh": [435], "bhandhlyp": [436],
}
MGGA_IDS = (202, 231)


def build():
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.oracle_functional.argtypes = [C.c_int, C.c_long, _dp, _dp, _dp, _dp, _dp]
        L.oracle_collocation.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, C.c_long, _dp,
                                         C.c_int, _dp]
        L.oracle_decay_cutoff.argtypes = [C.c_int, _ip, _ip, _ip, _dp, _dp, _dp, C.c_int,
                                          C.c_double, _dp]
        L.oracle_morton_leaves.argtypes = [C.c_long, _dp, C.c_long, C.c_long, C.c_long, _lp, _lp,
                                           _lp, _dp, _dp]
        L.oracle_morton_leaves.restype = C.c_long
        L.oracle_xc_build.argtypes = [C.c_int, _ip, _ip, _ip, _dp, _dp, _dp, C.c_int, C.c_long,
                                      _dp, _dp, _dp, C.c_int, _ip, _dp, C.c_double, C.c_double,
                                      C.c_long, C.c_long, C.c_long, C.c_int, C.c_long, _dp, _dp,
                                      _dp]
        _lib = L
    return _lib


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def functional(fid, rho, sigma=None):
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    n = len(rho)
    sig = np.ascontiguousarray(sigma if sigma is not None else np.zeros(n), dtype=np.float64)
    exc, vrho, vsig = np.zeros(n), np.zeros(n), np.zeros(n)
    rc = lib().oracle_functional(fid, n, _p(rho), _p(sig), _p(exc), _p(vrho), _p(vsig))
    if rc != 0:
        raise ValueError(f"unknown functional {fid}")
    return exc, vrho, vsig


def functional_mgga(fid, rho, sigma, tau):
    """Unpolarised meta-GGA at n points: exc (per particle), vrho, vsigma, vtau."""
    rho, sigma, tau = (np.ascontiguousarray(x, dtype=np.float64) for x in (rho, sigma, tau))
    n = len(rho)
    out = [np.zeros(n) for _ in range(4)]
    L = lib()
    L.oracle_functional_mgga.restype = C.c_int
    L.oracle_functional_mgga.argtypes = [C.c_int, C.c_long] + [_dp] * 7
    rc = L.oracle_functional_mgga(int(fid), n, _p(rho), _p(sigma), _p(tau),
                                  *[_p(x) for x in out])
    if rc != 0:
        raise ValueError(f"not a meta-GGA: {fid}")
    return tuple(out)


def functional_mgga_polarized(fid, ra, rb, saa, sab, sbb, ta, tb):
    """Polarised meta-GGA: exc (per particle), vrho (n x 2), vsigma (n x 3),
    vtau (n x 2)."""
    xs = [np.ascontiguousarray(x, dtype=np.float64) for x in (ra, rb, saa, sab, sbb, ta, tb)]
    n = len(xs[0])
    exc, vr, vs, vt = np.zeros(n), np.zeros((n, 2)), np.zeros((n, 3)), np.zeros((n, 2))
    L = lib()
    L.oracle_functional_mgga_polarized.restype = C.c_int
    L.oracle_functional_mgga_polarized.argtypes = [C.c_int, C.c_long] + [_dp] * 11
    rc = L.oracle_functional_mgga_polarized(int(fid), n, *[_p(x) for x in xs], _p(exc), _p(vr),
                                            _p(vs), _p(vt))
    if rc != 0:
        raise ValueError(f"not a meta-GGA: {fid}")
    return exc, vr, vs, vt


def collocation(l, pure, exps, coefs, origin, xyz, deriv=1):
    exps = np.ascontiguousarray(exps, dtype=np.float64)
    coefs = np.ascontiguousarray(coefs, dtype=np.float64)
    origin = np.ascontiguousarray(origin, dtype=np.float64)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    nf = 2 * l + 1 if pure else (l + 1) * (l + 2) // 2
    out = np.zeros(({0: 1, 1: 4, 2: 10}[int(deriv)], nf, len(xyz)))
    lib().oracle_collocation(l, int(pure), len(exps), _p(exps), _p(coefs), _p(origin), len(xyz),
                             _p(xyz), int(deriv), _p(out))
    return out


def _basis_arrays(basis):
    l, atom, nprim, exps, coefs = basis.arrays()
    off = np.zeros(len(l), dtype=np.int32)
    off[1:] = np.cumsum(nprim)[:-1]
    origin = np.array([s.origin for s in basis.shells], dtype=np.float64).ravel()
    return l, nprim, off, exps, coefs, origin


def decay_cutoff(basis, threshold=1e-10):
    l, nprim, off, exps, coefs, origin = _basis_arrays(basis)
    ext = np.zeros(len(l))
    lib().oracle_decay_cutoff(len(l), _p(l, _ip), _p(nprim, _ip), _p(off, _ip), _p(exps),
                              _p(coefs), _p(origin), int(basis.pure), threshold, _p(ext))
    return ext


def morton_leaves(points, target=128, min_leaf=32, max_leaf=256):
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    n = len(pts)
    perm = np.zeros(n, dtype=np.int64)
    off = np.zeros(n + 1, dtype=np.int64)
    cnt = np.zeros(n + 1, dtype=np.int64)
    cen = np.zeros(3 * (n + 1))
    rad = np.zeros(n + 1)
    nl = lib().oracle_morton_leaves(n, _p(pts), target, min_leaf, max_leaf, _p(perm, _lp),
                                    _p(off, _lp), _p(cnt, _lp), _p(cen), _p(rad))
    return perm, off[:nl], cnt[:nl], cen[:3 * nl].reshape(-1, 3), rad[:nl]


def xc_build(basis, points, weights, D, method, screen=1e-10, density_threshold=1e-10,
             leaf=(128, 32, 256), nthreads=0, leaf_stride=1, func_ids=None):
    """E_xc, V_xc (nbf x nbf) and the integrated density for mo.D = D."""
    l, nprim, off, exps, coefs, origin = _basis_arrays(basis)
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    nbf = basis.nbf()
    Df = np.asfortranarray(D, dtype=np.float64)
    ids = np.array(func_ids if func_ids is not None else METHODS[method.lower()], dtype=np.int32)
    coef = np.ones(len(ids))
    V = np.zeros((nbf, nbf), order="F")
    exc = C.c_double()
    nel = C.c_double()
    rc = lib().oracle_xc_build(len(l), _p(l, _ip), _p(nprim, _ip), _p(off, _ip), _p(exps),
                               _p(coefs), _p(origin), int(basis.pure), len(w), _p(pts), _p(w),
                               Df.ctypes.data_as(_dp), len(ids), _p(ids, _ip), _p(coef), screen,
                               density_threshold, leaf[0], leaf[1], leaf[2], nthreads,
                               leaf_stride, V.ctypes.data_as(_dp), C.byref(exc), C.byref(nel))
    if rc != 0:
        raise RuntimeError(f"oracle_xc_build failed ({rc})")
    return exc.value, V, nel.value


def xc_gradient(basis, points, weights, D, method, screen=1e-10, density_threshold=1e-10,
                leaf=(128, 32, 256), nthreads=0):
    """dE_xc/dR (natoms x 3, Hartree/Bohr) for mo.D = D, grid weights fixed
    (include/occ/dft/dft.h:599-749)."""
    l, nprim, off, exps, coefs, origin = _basis_arrays(basis)
    atom = np.array([s.atom for s in basis.shells], dtype=np.int32)
    natoms = len(basis.atoms())
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    Df = np.asfortranarray(D, dtype=np.float64)
    ids = np.array(METHODS[method.lower()], dtype=np.int32)
    coef = np.ones(len(ids))
    g = np.zeros(3 * natoms)
    L = lib()
    L.oracle_xc_gradient.restype = C.c_int
    rc = L.oracle_xc_gradient(len(l), _p(l, _ip), _p(nprim, _ip), _p(off, _ip), _p(exps),
                              _p(coefs), _p(origin), _p(atom, _ip), natoms, int(basis.pure),
                              len(w), _p(pts), _p(w), Df.ctypes.data_as(_dp), len(ids),
                              _p(ids, _ip), _p(coef), C.c_double(screen),
                              C.c_double(density_threshold), C.c_long(leaf[0]),
                              C.c_long(leaf[1]), C.c_long(leaf[2]), nthreads, _p(g))
    if rc != 0:
        raise RuntimeError(f"oracle_xc_gradient failed ({rc})")
    return g.reshape(natoms, 3)


def xc_gradient_unrestricted(basis, points, weights, D, method, screen=1e-10,
                             density_threshold=1e-10, leaf=(128, 32, 256), nthreads=0):
    """dE_xc/dR (natoms x 3) for OCC's unrestricted mo.D (2 nbf x nbf), grid
    weights fixed (include/occ/dft/dft.h:599-749, the Unrestricted branch)."""
    l, nprim, off, exps, coefs, origin = _basis_arrays(basis)
    atom = np.array([s.atom for s in basis.shells], dtype=np.int32)
    natoms = len(basis.atoms())
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    Df = np.asfortranarray(D, dtype=np.float64)
    if Df.shape != (2 * basis.nbf(), basis.nbf()):
        raise ValueError("D must be 2 nbf x nbf")
    ids = np.array(METHODS[method.lower()], dtype=np.int32)
    coef = np.ones(len(ids))
    g = np.zeros(3 * natoms)
    L = lib()
    L.oracle_xc_gradient_unrestricted.restype = C.c_int
    rc = L.oracle_xc_gradient_unrestricted(
        len(l), _p(l, _ip), _p(nprim, _ip), _p(off, _ip), _p(exps), _p(coefs), _p(origin),
        _p(atom, _ip), natoms, int(basis.pure), len(w), _p(pts), _p(w), Df.ctypes.data_as(_dp),
        len(ids), _p(ids, _ip), _p(coef), C.c_double(screen), C.c_double(density_threshold),
        C.c_long(leaf[0]), C.c_long(leaf[1]), C.c_long(leaf[2]), nthreads, _p(g))
    if rc != 0:
        raise RuntimeError(f"oracle_xc_gradient_unrestricted failed ({rc})")
    return g.reshape(natoms, 3)


def functional_polarized(fid, ra, rb, saa=None, sab=None, sbb=None):
    """Polarised functional at n points: exc (per particle), vrho (n x 2),
    vsigma (n x 3; zeros for an LDA)."""
    ra = np.ascontiguousarray(ra, dtype=np.float64)
    rb = np.ascontiguousarray(rb, dtype=np.float64)
    n = len(ra)
    z = np.zeros(n)
    s = [np.ascontiguousarray(x, dtype=np.float64) if x is not None else z
         for x in (saa, sab, sbb)]
    exc = np.zeros(n)
    v = [np.zeros(n) for _ in range(5)]
    L = lib()
    L.oracle_functional_polarized.restype = C.c_int
    L.oracle_functional_polarized.argtypes = [C.c_int, C.c_long] + [_dp] * 11
    rc = L.oracle_functional_polarized(int(fid), n, _p(ra), _p(rb), _p(s[0]), _p(s[1]),
                                       _p(s[2]), _p(exc), *[_p(x) for x in v])
    if rc != 0:
        raise ValueError(f"unknown functional {fid}")
    return exc, np.stack(v[:2], axis=1), np.stack(v[2:], axis=1)


def xc_build_unrestricted(basis, points, weights, D, method, screen=1e-10,
                          density_threshold=1e-10, leaf=(128, 32, 256), nthreads=0):
    """E_xc, V (2 nbf x nbf, alpha block above beta) and the integrated
    (alpha, beta) densities for OCC's unrestricted mo.D (2 nbf x nbf)."""
    l, nprim, off, exps, coefs, origin = _basis_arrays(basis)
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    nbf = basis.nbf()
    Df = np.asfortranarray(D, dtype=np.float64)
    if Df.shape != (2 * nbf, nbf):
        raise ValueError("D must be 2 nbf x nbf")
    ids = np.array(METHODS[method.lower()], dtype=np.int32)
    coef = np.ones(len(ids))
    V = np.zeros((2 * nbf, nbf), order="F")
    exc = C.c_double()
    nel = np.zeros(2)
    L = lib()
    L.oracle_xc_build_unrestricted.restype = C.c_int
    L.oracle_xc_build_unrestricted.argtypes = [
        C.c_int, _ip, _ip, _ip, _dp, _dp, _dp, C.c_int, C.c_long, _dp, _dp, _dp, C.c_int, _ip,
        _dp, C.c_double, C.c_double, C.c_long, C.c_long, C.c_long, C.c_int, _dp, _dp, _dp]
    rc = L.oracle_xc_build_unrestricted(
        len(l), _p(l, _ip), _p(nprim, _ip), _p(off, _ip), _p(exps), _p(coefs), _p(origin),
        int(basis.pure), len(w), _p(pts), _p(w), Df.ctypes.data_as(_dp), len(ids), _p(ids, _ip),
        _p(coef), C.c_double(screen), C.c_double(density_threshold), C.c_long(leaf[0]),
        C.c_long(leaf[1]), C.c_long(leaf[2]), nthreads, V.ctypes.data_as(_dp), C.byref(exc),
        _p(nel))
    if rc != 0:
        raise RuntimeError(f"oracle_xc_build_unrestricted failed ({rc})")
    return exc.value, V, nel


NLC_GRID = dict(max_angular_points=110, min_angular_points=50, radial_points=50,
                radial_precision=1e-7)  # src/dft/nonlocal_correlation.cpp set_integration_grid


def vv10_kernel(points, weights, rho, sigma, b=6.0, c=0.01, nthreads=0):
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    r = np.ascontiguousarray(rho, dtype=np.float64)
    s = np.ascontiguousarray(sigma, dtype=np.float64)
    n = len(w)
    out = [np.zeros(n) for _ in range(3)]
    L = lib()
    L.oracle_vv10_kernel.argtypes = [C.c_long, _dp, _dp, _dp, _dp, C.c_double, C.c_double,
                                     C.c_int, _dp, _dp, _dp]
    L.oracle_vv10_kernel(n, _p(pts), _p(w), _p(r), _p(s), b, c, nthreads, *[_p(x) for x in out])
    return out


def nlc_vv10(basis, points, weights, D, b=6.0, c=0.01, nthreads=0, want_V=True):
    """Energy and V (nbf x nbf) of VV10 on the given NLC grid (in grid order)."""
    l, nprim, off, exps, coefs, origin = _basis_arrays(basis)
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    nbf = basis.nbf()
    Df = np.asfortranarray(D, dtype=np.float64)
    V = np.zeros((nbf, nbf), order="F") if want_V else None
    e = C.c_double()
    L = lib()
    L.oracle_nlc_vv10.restype = C.c_int
    L.oracle_nlc_vv10.argtypes = [C.c_int, _ip, _ip, _ip, _dp, _dp, _dp, C.c_int, C.c_long, _dp,
                                  _dp, _dp, C.c_double, C.c_double, C.c_int, _dp, _dp]
    rc = L.oracle_nlc_vv10(len(l), _p(l, _ip), _p(nprim, _ip), _p(off, _ip), _p(exps),
                           _p(coefs), _p(origin), int(basis.pure), len(w), _p(pts), _p(w),
                           Df.ctypes.data_as(_dp), b, c, nthreads,
                           V.ctypes.data_as(_dp) if want_V else None, C.byref(e))
    if rc != 0:
        raise RuntimeError("oracle_nlc_vv10 failed")
    return e.value, V
