"""The device-side error words reach the caller.  Every wait of a tensor-core kernel on an mbarrier is
bounded; when it runs out the kernel sets a timeout word and returns, and the next mlg_sync or vortex
step must report MLG_ETIMEOUT, clear the word, and leave the context usable.  The wait is made to run
out on purpose through mlg_selftest_bounded_wait (one thread waiting on an mbarrier that nothing
arrives at, for about a millisecond): nothing faults, traps or hangs."""
import numpy as np
import pytest

from helpers import params

pytestmark = pytest.mark.gpu

MLG_ETIMEOUT = 13
LIMIT = 2_000_000   # SM clocks, about a millisecond


def test_wait_that_runs_out_reaches_mlg_sync():
    from mlegs_gb300 import fields
    from mlegs_gb300.kit import Kit, load
    L = load()
    k = Kit(params("c1"))
    e = fields.spectral_noise(k.params, k.dims, 3, amp=1.0, decay=0.3)

    def round_trip():
        s = k.scalar(e, 0.0, "FFF")
        k.trans(s, "PPP")
        k.trans(s, "FFF")
        out = s.e
        s.free()
        return out

    before = round_trip()
    assert L.mlg_selftest_bounded_wait(LIMIT, 1) == 0
    assert L.mlg_sync() == 0, "a wait that succeeds must leave no error"
    assert L.mlg_selftest_bounded_wait(LIMIT, 0) == 0
    assert L.mlg_sync() == MLG_ETIMEOUT
    assert b"bounded device-side wait" in L.mlg_last_error()
    assert L.mlg_sync() == 0, "the timeout word is cleared once reported"
    # the context is still usable: the same round trip gives the same bytes
    assert np.array_equal(round_trip(), before)
    k.close()


def test_wait_that_runs_out_reaches_vortex_run():
    from mlegs_gb300 import vortex
    from mlegs_gb300.kit import Kit, MlgError, load
    L = load()
    k = Kit(params("c1"))
    st = vortex.VortexState(k)
    vortex.qvort_init(k, st, q=4.0)
    k.advection_rhs(st.psi, st.chi, st.nlpsi, st.nlchi, st.uz)
    assert L.mlg_selftest_bounded_wait(LIMIT, 0) == 0
    with pytest.raises(MlgError) as ei:
        k.vortex_run(*st.args(), 1e-3, 2, st.gains)
    assert ei.value.code == MLG_ETIMEOUT
    k.vortex_run(*st.args(), 1e-3, 2, st.gains)   # reported once, then clear
    assert np.isfinite(st.psi.e).all()
    st.free()
    k.close()


def test_selftest_rejects_out_of_range_limit():
    from mlegs_gb300.kit import Kit, load
    L = load()
    k = Kit(params("c1"))
    assert L.mlg_selftest_bounded_wait(-1, 0) == 1
    assert L.mlg_selftest_bounded_wait(3_000_000_000, 0) == 1
    assert L.mlg_sync() == 0
    k.close()
