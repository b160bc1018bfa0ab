"""The CPU restatement (oracle/) against the reference's rollouts of the benchmark workloads
(tests/workload_data.py): the portable build within tolerance, discrete state, ball-hit counters and
events equal, up to the kickoff resets (which only the reference and the CUDA path implement)."""
import pytest

from golden_data import check_continuous
from workload_data import GROUPS, check_arena, load_workload, play_cpu


@pytest.mark.parametrize("name", GROUPS)
def test_portable_restatement_follows_the_reference(name):
    wl = load_workload(name)
    step = 4 if name != "hits" else 1  # a sample of the larger groups keeps the CPU suite short
    for si in range(0, wl.S, step):
        snaps, events = play_cpu("oracle", wl, si)
        check_arena(wl, si, snaps, events, check_continuous, f"oracle {name}")


@pytest.mark.skipif(__import__("platform").machine() not in ("x86_64", "AMD64"), reason="SSE emulation build is x86 only")
@pytest.mark.parametrize("name", GROUPS)
def test_sse_restatement_bit_exact_on_the_workloads(name):
    """The restatement's SSE build reproduces the reference's car and ball states bit for bit after
    1 and 8 ticks on the sampled arenas."""
    wl = load_workload(name)
    for si in range(0, wl.S, 8 if name != "hits" else 1):
        snaps, _ = play_cpu("oracle_sse", wl, si, ticks=8)
        for t in (1, 8):
            cars, ball, _ = snaps[t - 1]
            for f in ("pos", "vel", "ang_vel", "rot_mat"):
                assert cars[f].tobytes() == wl.cars_at(si, t)[f].tobytes(), f"{name} arena {si} tick {t} {f}"
            for f in ("pos", "vel", "ang_vel"):
                assert ball[f].tobytes() == wl.ball_at(si, t)[f].tobytes(), f"{name} arena {si} tick {t} ball {f}"
