"""The bounded waits of the tensor-core pipeline, made to run out on purpose.

occ_xc_set_wait_limit(ctx, 0) makes every pipeline wait of the persistent
density and V_xc kernels give up at once: each CTA sets the build's error
flag, waits for its own bulk copies and MMAs in flight, frees its tensor
memory and returns.  The call reports OCC_XC_ERR_TIMEOUT; with the default
bound restored, the next build on the same molecule and context equals the
FP64 build within the mixed path's bars."""
import numpy as np
import pytest

import occ_gb300 as og
from occ_gb300 import workloads as wl
from helpers import TOL_E_MIXED, TOL_V_MIXED

pytestmark = pytest.mark.gpu
DEFAULT_POLLS = 1 << 24


@pytest.mark.parametrize("method", ["pbe", "lda"])
def test_wait_running_out_reports_timeout_then_builds_recover(method):
    mol = wl.water_cluster(4, box=5.0, seed=1)
    b = wl.basis_for(mol, "def2-svp")
    D = wl.random_density(b.nbf(), 20, seed=2)
    dft = og.DFT(method, b)
    V64 = dft.compute_vxc(D, og.FP64)
    e64 = dft.exchange_correlation_energy()
    dft.compute_vxc(D, og.MIXED)  # workspace and AO values in place
    lib = dft.ctx.lib
    assert lib.occ_xc_set_wait_limit(dft.ctx.h, 0) == 0
    try:
        with pytest.raises(og.XCError) as err:
            dft.compute_vxc(D, og.MIXED)
        assert "(-5)" in str(err.value)
    finally:
        assert lib.occ_xc_set_wait_limit(dft.ctx.h, DEFAULT_POLLS) == 0
    for _ in range(2):
        V = dft.compute_vxc(D, og.MIXED)
        assert abs(dft.exchange_correlation_energy() - e64) <= TOL_E_MIXED
        assert np.max(np.abs(V - V64)) <= TOL_V_MIXED
