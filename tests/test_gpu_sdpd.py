"""GPU SDPD parity: the particle step on the GPU against the oracle and the
compiled reference engine.

The GPU kernels and the oracle (oracle/sdpd_oracle_impl.h) evaluate the
same operations in the same order without FMA contraction, so states are
compared bit for bit in both precisions.  Against the reference engine
(tests/golden/sdpd_small.npz) the tolerance is 1e-12 absolute on positions
and densities and 1e-9 norm-wise relative on velocities (summation order of
tied neighbours differs).
"""
import numpy as np
import pytest

from spatialpy_gb300 import scenario as S

from .conftest import golden

pytestmark = pytest.mark.gpu


def _engine(sc, prec):
    from spatialpy_gb300.engine import Engine
    return Engine(sc, sdpd_precision=prec)


@pytest.mark.parametrize("div", [8, 16])
@pytest.mark.parametrize("prec,mode", [("f64", 2), ("f32", 6)])
def test_sdpd_bitexact_vs_oracle(oracle_lib, div, prec, mode):
    sc = S.config_dam_break(spacing_div=div, num_steps=41)
    st = oracle_lib.SdpdState(sc)
    with _engine(sc, prec) as eng:
        done = 0
        for n in (1, 5, 21, 41):
            eng.sdpd_advance(n - done)
            oracle_lib.sdpd(sc, st, n - done, prec, mode)
            done = n
            x, v, rho = eng.particles(0)
            np.testing.assert_array_equal(x, st.x, err_msg=f"x step {n}")
            np.testing.assert_array_equal(v, st.v, err_msg=f"v step {n}")
            np.testing.assert_array_equal(rho, st.rho, err_msg=f"rho step {n}")
        cnt, idx, dist, dw, _ = eng.neighbors(0, 64)
        np.testing.assert_array_equal(cnt, st.nbr_count)


def test_sdpd_f64_vs_reference_golden():
    g = golden("sdpd_small.npz")
    sc = S.config_dam_break(spacing_div=int(g["spacing_div"]), num_steps=41)
    with _engine(sc, "f64") as eng:
        done = 0
        for n in (1, 5, 21, 41):
            eng.sdpd_advance(n - done)
            done = n
            x, v, rho = eng.particles(0)
            rv = g[f"{n}/v"]
            assert np.abs(x - g[f"{n}/x"]).max() <= 1e-12
            assert np.linalg.norm(v - rv) <= 1e-9 * max(np.linalg.norm(rv), 1e-30)
            assert np.abs(rho - g[f"{n}/rho"]).max() <= 1e-12


def test_sdpd_f32_tracks_f64_over_1000_steps():
    """FP32 state against FP64 after 1,000 steps, norm-wise relative:
    positions within 1e-5; velocities within 1e-3 (3e-4 measured: velocities
    start near zero and early rounding differences persist)."""
    sc = S.config_dam_break(spacing_div=8, num_steps=1000)
    with _engine(sc, "f64") as a, _engine(sc, "f32") as b:
        a.sdpd_advance(1000)
        b.sdpd_advance(1000)
        xa, va, ra = a.particles(0)
        xb, vb, rb = b.particles(0)
    assert np.linalg.norm(xa - xb) <= 1e-5 * np.linalg.norm(xa)
    assert np.linalg.norm(va - vb) <= 1e-3 * np.linalg.norm(va)
    assert np.abs(ra - rb).max() <= 1e-4


def test_sdpd_neighbor_sets_match_oracle_after_motion(oracle_lib):
    """Neighbour sets of moved particles (query at the moved position, points
    at the start of the step) equal the oracle's after 30 steps."""
    sc = S.config_dam_break(spacing_div=16, num_steps=30)
    st = oracle_lib.SdpdState(sc)
    oracle_lib.sdpd(sc, st, 30, "f64", 2)
    with _engine(sc, "f64") as eng:
        eng.sdpd_advance(30)
        cnt, idx, dist, dw, _ = eng.neighbors(0, 64)
    np.testing.assert_array_equal(cnt, st.nbr_count)
    # moved fluid particles carry their own start-of-step point
    fluid = np.nonzero(sc.fixed == 0)[0]
    assert all(i in idx[i, :cnt[i]] for i in fluid[:200])
