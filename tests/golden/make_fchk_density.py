"""Generate two density fixtures from the Gaussian formatted checkpoints
embedded in the reference's tests (tests/wavefunction_io_tests.cpp, read as
text):

* water_rhf_631gdp.npz: a converged RHF density of water in a pure
  6-31G(d,p) basis (24 AOs), `pure_fchk_contents`;
* water_uhf_321g_fchk.npz: the converged water 3-21G UHF with 5 alpha = 5
  beta electrons, `unrestricted_fchk_contents` (a closed shell, so its alpha
  density is the RHF density; SCF energy -75.585325704292 Ha, RMS density
  change 6e-10), which pins tests/golden/make_hf_density.py at its geometry;

both in OCC's conventions:

* shells as OCC's FchkReader::basis_set builds them (src/qm/io/fchkreader.cpp
  :327-395): SP shells split into an s and a p shell on the same exponents,
  contraction coefficients as stored (normalised later by
  incorporate_shell_norm, here occ_xc_normalize_shell);
* AO order converted from Gaussian's to OCC's as
  from_gaussian_order_spherical does (src/qm/io/conversion.cpp:174-207):
  p (x, y, z) -> (y, z, x); l >= 2: OCC's m = -l..l from Gaussian's
  0, +1, -1, +2, -2, ...;
* mo.D = C_occ C_occ^T of the 5 occupied alpha orbitals (restricted), and
  the file's "Total SCF Density" (= 2 mo.D) reordered the same way as a
  cross-check of the conversion.

usage: python tests/golden/make_fchk_density.py [path of wavefunction_io_tests.cpp]
(default: $OCC_REFERENCE/tests/wavefunction_io_tests.cpp, OCC_REFERENCE being
the reference checkout)
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(os.environ.get("OCC_REFERENCE", "/root/reference"),
                   "tests", "wavefunction_io_tests.cpp")


def fchk_text(src, name="pure_fchk_contents"):
    s = open(src).read()
    m = re.search(name + r'\s*=\s*R"\((.*?)\)"', s, re.S)
    if not m:
        raise SystemExit(name + " not found")
    return m.group(1)


def field(text, name):
    """Values of an array field ('... R   N=  k' or '... I   N=  k'), or a scalar."""
    lines = text.splitlines()
    for i, ln in enumerate(lines):
        if ln.startswith(name):
            kind = ln[43]
            if "N=" in ln:
                n = int(ln.split("N=")[1])
                vals = []
                j = i + 1
                while len(vals) < n:
                    vals += lines[j].split()
                    j += 1
                conv = int if kind == "I" else float
                return np.array([conv(v) for v in vals[:n]])
            return (int if kind == "I" else float)(ln.split()[-1])
    raise KeyError(name)


def gaussian_to_occ(l, pure=True):
    """perm[k] = Gaussian index of OCC's function k within a shell."""
    if l == 1:
        return [1, 2, 0]  # OCC (y, z, x) from Gaussian (x, y, z)
    if l == 0 or not pure:
        return list(range(2 * l + 1 if pure else (l + 1) * (l + 2) // 2))
    out = []
    for m in range(-l, l + 1):
        out.append(0 if m == 0 else (2 * m - 1 if m > 0 else -2 * m))
    return out


def convert(t):
    """Basis, OCC-ordered alpha density mo.D = C_occ C_occ^T and the file's
    Total SCF Density (reordered) of one formatted checkpoint."""
    Z = field(t, "Atomic numbers")
    xyz = field(t, "Current cartesian coordinates").reshape(-1, 3)  # Bohr
    types = field(t, "Shell types")
    nprim = field(t, "Number of primitives per shell")
    sh_atom = field(t, "Shell to atom map") - 1
    exps = field(t, "Primitive exponents")
    coefs = field(t, "Contraction coefficients")
    spc = field(t, "P(S=P) Contraction coefficients")
    nbf = field(t, "Number of basis functions")
    nalpha = field(t, "Number of alpha electrons")
    C = field(t, "Alpha MO coefficients").reshape(nbf, nbf).T  # column k = MO k
    tri = field(t, "Total SCF Density")
    P = np.zeros((nbf, nbf))
    P[np.tril_indices(nbf)] = tri
    P = P + P.T - np.diag(np.diag(P))

    shells = []  # (l, atom, exps, coefs)
    perm = []
    off = 0
    bf = 0
    for st, n, a in zip(types, nprim, sh_atom):
        e = exps[off:off + n]
        if st == -1:  # SP
            shells.append((0, a, e, coefs[off:off + n]))
            shells.append((1, a, e, spc[off:off + n]))
            perm += [bf]
            perm += [bf + 1 + k for k in gaussian_to_occ(1)]
            bf += 4
        else:
            l = abs(st)
            shells.append((l, a, e, coefs[off:off + n]))
            perm += [bf + k for k in gaussian_to_occ(l)]
            bf += 2 * l + 1
        off += n
    assert bf == nbf
    perm = np.array(perm)
    C_occ = C[perm, :nalpha]
    D = C_occ @ C_occ.T
    P_occ = P[np.ix_(perm, perm)]
    return dict(
        Z=Z, xyz_bohr=xyz, shell_l=np.array([s[0] for s in shells]),
        shell_atom=np.array([s[1] for s in shells]),
        shell_nprim=np.array([len(s[2]) for s in shells]),
        exponents=np.concatenate([s[2] for s in shells]),
        coefficients=np.concatenate([s[3] for s in shells]),
        D=D, total_scf_density=P_occ, nelec=np.array(2 * nalpha),
        scf_energy=np.array(field(t, "SCF Energy")))


def main(src):
    # pure 6-31G(d,p) RHF
    d = convert(fchk_text(src, "pure_fchk_contents"))
    err = np.max(np.abs(2 * d["D"] - d["total_scf_density"]))
    assert err < 1e-6, err
    np.savez_compressed(os.path.join(HERE, "water_rhf_631gdp.npz"), **d)
    print("wrote water_rhf_631gdp.npz: nbf", d["D"].shape[0], "max|2D - P|", err)
    # 3-21G UHF with 5 alpha = 5 beta electrons (a closed shell): its alpha
    # density pins the small RHF of make_hf_density.py at this geometry
    d = convert(fchk_text(src, "unrestricted_fchk_contents"))
    err = np.max(np.abs(2 * d["D"] - d["total_scf_density"]))
    assert err < 1e-6, err
    np.savez_compressed(os.path.join(HERE, "water_uhf_321g_fchk.npz"), **d)
    print("wrote water_uhf_321g_fchk.npz: nbf", d["D"].shape[0], "max|2D - P|", err)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else SRC)
