"""The C++ host interface (include/occ_xc.hpp, shaped like occ::dft::DFT):
tests/cpp/test_dft.cpp is compiled against the in-tree library and run on
the converged water density; the oracle's E_xc per method is its reference."""
import os
import subprocess

import numpy as np
import pytest

import occ_gb300 as og
import oracle
from helpers import host_grid
from test_fchk_density import HERE

ROOT = os.path.dirname(HERE)


def _compile(out):
    lib_dir = os.path.dirname(og.library_path())
    cmd = ["g++", "-std=c++17", "-O2", os.path.join(HERE, "cpp", "test_dft.cpp"),
           "-I", os.path.join(ROOT, "include"), "-L", lib_dir, "-locc_xc",
           "-Wl,-rpath," + lib_dir, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_cpp_header_compiles(tmp_path):
    """The header and the test program build against the library (no GPU)."""
    og.library()
    _compile(str(tmp_path / "test_dft"))


@pytest.mark.gpu
def test_cpp_dft_interface(tmp_path):
    f = np.load(os.path.join(HERE, "golden", "water_rhf_631gdp.npz"))
    from test_fchk_density import fchk_case
    b, D, nelec = fchk_case()
    P, W = host_grid(b)
    lines = [str(len(f["Z"]))]
    lines += [f"{int(z)} {float(x)!r} {float(y)!r} {float(w)!r}"
              for z, (x, y, w) in zip(f["Z"], f["xyz_bohr"])]
    lines.append(str(len(f["shell_l"])))
    off = 0
    for l, a, n in zip(f["shell_l"], f["shell_atom"], f["shell_nprim"]):
        prims = " ".join(f"{float(e)!r} {float(c)!r}"
                         for e, c in zip(f["exponents"][off:off + n],
                                         f["coefficients"][off:off + n]))
        lines.append(f"{int(l)} {int(a)} {int(n)} {prims}")
        off += n
    lines.append(f"1 {D.shape[0]} {nelec}")
    lines.append(" ".join(repr(float(x)) for x in np.asfortranarray(D).ravel(order="F")))
    for method in ("lda", "pbe", "b3lyp"):
        e_ref, _, _ = oracle.xc_build(b, P, W, D, method)
        lines.append(f"{method} {float(e_ref)!r}")
    for method in ("lda", "pbe"):
        g_ref = oracle.xc_gradient(b, P, W, D, method)
        lines.append(f"grad {method} " + " ".join(repr(float(x)) for x in g_ref.ravel()))
    inp = tmp_path / "input.txt"
    inp.write_text("\n".join(lines) + "\n")
    exe = _compile(str(tmp_path / "test_dft"))
    r = subprocess.run([exe, str(inp)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
