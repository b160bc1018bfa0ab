"""The CPU restatement (oracle/) against the reference's own outputs.

The golden rollouts were produced by the reference RocketSim built from its own
sources (tests/golden/make_golden.py).  The restatement compiled with the SSE
reciprocal-square-root emulation (x86 only) must reproduce them bit for bit; the
portable build (exact square root, the arithmetic the CUDA code uses) within the
stated tolerance, with identical discrete state.
"""
import platform

import numpy as np
import pytest

from golden_data import check_continuous
from scenarios import cpu_snapshot, discrete_car, discrete_pads, run_cpu


def play(kind, golden, si, ticks=120):
    sc = golden.scenarios[si]
    snaps = []
    a, ids = run_cpu(kind, sc, ticks, record=lambda t, a, ids: snaps.append(cpu_snapshot(a, ids)))
    a.close()
    return snaps


def check_discrete(golden, si, snaps, exact_until):
    for t in range(min(exact_until, len(snaps))):
        cars, ball, pads = snaps[t]
        np.testing.assert_array_equal(discrete_car(cars).astype(np.float32), golden.disc_cars(si)[t],
                                      err_msg=f"scenario {si} tick {t + 1}: car discrete state")
        np.testing.assert_array_equal(discrete_pads(pads).astype(np.float32), golden.disc_pads(si)[t],
                                      err_msg=f"scenario {si} tick {t + 1}: pad state")


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"), reason="SSE emulation build is x86 only")
def test_sse_restatement_bit_exact(golden):
    for si in range(golden.S):
        snaps = play("oracle_sse", golden, si, 8)
        for t in (1, 8):
            cars, ball, _ = snaps[t - 1]
            ref_cars, ref_ball = golden.cars_at(si, t), golden.ball_at(si, t)
            for f in ("pos", "vel", "ang_vel", "rot_mat"):
                assert cars[f].tobytes() == ref_cars[f].tobytes(), f"scenario {si} tick {t} {f}"
                if f != "rot_mat":
                    assert ball[f].tobytes() == ref_ball[f].tobytes(), f"scenario {si} tick {t} ball {f}"


def test_portable_restatement_within_tolerance(golden):
    for si in range(golden.S):
        snaps = play("oracle", golden, si, 120)
        for t in (1, 8):
            cars, ball, _ = snaps[t - 1]
            check_continuous(cars, ball, golden.cars_at(si, t), golden.ball_at(si, t), t, f"scenario {si}")
        check_discrete(golden, si, snaps, 120)


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"), reason="SSE emulation build is x86 only")
def test_sse_restatement_bit_exact_through_epa(golden):
    """Scenarios where the reference runs Bullet's GJK-EPA penetration solver: the restatement
    follows it bit for bit over every one of the 120 ticks (the reference run live here)."""
    import os
    ref_so = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "librsref.so")
    if not os.path.exists(ref_so):
        pytest.skip("reference library not built here")
    epa_scenarios = [si for si in range(golden.S) if golden.epa_tick(si) >= 0]
    assert epa_scenarios
    for si in epa_scenarios:
        ref = play("ref", golden, si, 120)
        got = play("oracle_sse", golden, si, 120)
        for t in range(120):
            for f in ("pos", "vel", "ang_vel", "rot_mat"):
                assert got[t][0][f].tobytes() == ref[t][0][f].tobytes(), f"scenario {si} tick {t + 1} car {f}"
            for f in ("pos", "vel", "ang_vel"):
                assert got[t][1][f].tobytes() == ref[t][1][f].tobytes(), f"scenario {si} tick {t + 1} ball {f}"
