"""XC nuclear gradient, dE_xc/dR with the grid held fixed (OCC's
DFT::compute_xc_gradient, include/occ/dft/dft.h:599-749 and
src/dft/dft_gradient_kernels.cpp:472-595).

The oracle's gradient is pinned as the derivative of the oracle's E_xc (itself
pinned to the reference's golden vectors): central differences over shifts of
one atom's basis functions, grid fixed, on the converged water density.  The
screened gradient matches the dense one as the reference's
"DFT XC screening matches dense (gradient)" test requires (tests/dft_tests.cpp
:904-931)."""
import numpy as np
import pytest

import occ_gb300 as og
import oracle
from helpers import host_grid
from test_fchk_density import fchk_case


def _shifted(b, atom, axis, h):
    shells = []
    for s in b.shells:
        o = np.array(s.origin, dtype=np.float64).copy()
        if s.atom == atom:
            o[axis] += h
        shells.append(og.Shell(s.l, s.atom, o, s.exponents, s.coefficients))
    nb = og.AOBasis(b.atoms(), shells, b.name)
    nb.set_pure(b.pure)
    return nb


@pytest.mark.parametrize("method", ["lda", "pbe"])
def test_oracle_gradient_is_derivative_of_exc(method):
    b, D, _ = fchk_case()
    P, W = host_grid(b)
    g = oracle.xc_gradient(b, P, W, D, method, screen=1e-14)
    h = 1e-4
    for atom in range(3):
        for axis in range(3):
            ep = oracle.xc_build(_shifted(b, atom, axis, h), P, W, D, method, screen=1e-14)[0]
            em = oracle.xc_build(_shifted(b, atom, axis, -h), P, W, D, method, screen=1e-14)[0]
            assert abs(g[atom, axis] - (ep - em) / (2 * h)) < 1e-7, (atom, axis)


def test_oracle_gradient_screened_matches_dense():
    b, D, _ = fchk_case()
    P, W = host_grid(b)
    gs = oracle.xc_gradient(b, P, W, D, "pbe", screen=1e-10)
    gd = oracle.xc_gradient(b, P, W, D, "pbe", screen=0.0)
    assert np.max(np.abs(gs - gd)) < 1e-8
