"""Generate the golden fixtures of the CPU test suite from the reference's own
sources, compiled unmodified into oracle/_ref/libref.so (`make -C oracle ref`
on a machine that has the reference tree):

lebedev_ref.npz   Lebedev rules of the reference table (src/numint/lebedev.cpp)
                  for every point count up to 302: key n<count> -> (n, 4) x,y,z,w
gau2grid_ref.npz  AO values and gradients from gau2grid (src/3rdparty/gau2grid,
                  the collocation OCC's src/gto/gto.cpp:212-287 calls) for
                  l = 0..4, pure and Cartesian, seeded points and primitives,
                  scaled by OCC's common_fac (src/gto/gto.cpp:7-16)
gau2grid_deriv2_ref.npz  the same with second derivatives (xx, xy, xz, yy,
                  yz, zz), as the XC gradient evaluates them

usage: python tests/golden/make_golden.py
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref", "libref.so")
ORDERS = [6, 14, 26, 38, 50, 74, 86, 110, 146, 170, 194, 230, 266, 302]
GG_SPHERICAL_CCA, GG_CARTESIAN_CCA = 300, 400


def common_fac(l, pure):
    if l == 0:
        return 0.282094791773878143
    if l == 1:
        return 0.488602511902919921
    return np.sqrt((2 * l + 1) / (4 * np.pi)) if pure else 1.0


def main():
    lib = C.CDLL(REF)
    dp = C.POINTER(C.c_double)
    out = {}
    for n in ORDERS:
        a = np.zeros((n, 4))
        assert lib.ref_lebedev(n, a.ctypes.data_as(dp)) == n
        out[f"n{n}"] = a
    np.savez_compressed(os.path.join(HERE, "lebedev_ref.npz"), **out)

    rng = np.random.default_rng(2024)
    gg = {}
    for pure in (1, 0):
        for l in range(5):
            npt, nprim = 40, 3
            xyz = rng.normal(size=(npt, 3)) * 1.3
            A = rng.normal(size=3) * 0.5
            exps = np.sort(rng.uniform(0.1, 8.0, nprim))[::-1].copy()
            coefs = rng.uniform(0.2, 1.0, nprim)
            nf = 2 * l + 1 if pure else (l + 1) * (l + 2) // 2
            vals = np.zeros((4, nf, npt))
            lib.gg_collocation_deriv1(
                C.c_int(l), C.c_ulong(npt), xyz.ctypes.data_as(dp), C.c_ulong(3), C.c_int(nprim),
                coefs.ctypes.data_as(dp), exps.ctypes.data_as(dp), A.ctypes.data_as(dp),
                C.c_int(GG_SPHERICAL_CCA if pure else GG_CARTESIAN_CCA),
                vals[0].ctypes.data_as(dp), vals[1].ctypes.data_as(dp),
                vals[2].ctypes.data_as(dp), vals[3].ctypes.data_as(dp))
            key = f"{'pure' if pure else 'cart'}_l{l}"
            gg[key + "_xyz"] = xyz
            gg[key + "_A"] = A
            gg[key + "_exps"] = exps
            gg[key + "_coefs"] = coefs
            gg[key + "_vals"] = vals * common_fac(l, pure)
    np.savez_compressed(os.path.join(HERE, "gau2grid_ref.npz"), **gg)

    # second derivatives (gg_collocation_deriv2: phi, x, y, z, xx, xy, xz,
    # yy, yz, zz), the AO Hessians of the XC gradient (dft.h:628-631)
    rng = np.random.default_rng(2025)
    g2 = {}
    for pure in (1, 0):
        for l in range(5):
            npt, nprim = 40, 3
            xyz = rng.normal(size=(npt, 3)) * 1.3
            A = rng.normal(size=3) * 0.5
            exps = np.sort(rng.uniform(0.1, 8.0, nprim))[::-1].copy()
            coefs = rng.uniform(0.2, 1.0, nprim)
            nf = 2 * l + 1 if pure else (l + 1) * (l + 2) // 2
            vals = np.zeros((10, nf, npt))
            lib.gg_collocation_deriv2(
                C.c_int(l), C.c_ulong(npt), xyz.ctypes.data_as(dp), C.c_ulong(3), C.c_int(nprim),
                coefs.ctypes.data_as(dp), exps.ctypes.data_as(dp), A.ctypes.data_as(dp),
                C.c_int(GG_SPHERICAL_CCA if pure else GG_CARTESIAN_CCA),
                *[vals[q].ctypes.data_as(dp) for q in range(10)])
            key = f"{'pure' if pure else 'cart'}_l{l}"
            g2[key + "_xyz"] = xyz
            g2[key + "_A"] = A
            g2[key + "_exps"] = exps
            g2[key + "_coefs"] = coefs
            g2[key + "_vals"] = vals * common_fac(l, pure)
    np.savez_compressed(os.path.join(HERE, "gau2grid_deriv2_ref.npz"), **g2)


if __name__ == "__main__":
    main()
