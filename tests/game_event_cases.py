"""Scripts driving GameEventTracker through shots, goals and saves, run the same way on the reference
(tests/golden/make_game_event_golden.py) and on a batch (tests/test_gpu_game_events.py).

Each script acts on one soccar arena with four cars (teams blue, orange, blue, orange; ids 1-4, at
their respawn spots, away from the ball's path) and a tracker:
  ("ball", (x, y, z), (vx, vy, vz))  set the ball's state (the tick count since a state set restarts)
  ("hit", car_id, ticks_ago)          mark the car's last ball touch `ticks_ago` ticks before now
  ("car", car_id, (x, y, z))          put the car there, at rest on its wheels, facing +y
  ("step", k)                          play k ticks with no input
  ("update",)                          GameEventTracker::Update, its event recorded
  ("reset",)                           ResetPersistentInfo
"""
from __future__ import annotations

TEAMS = [0, 1, 0, 1]


def _ticks(n, k):
    out = []
    for _ in range(n):
        out += [("step", k), ("update",)]
    return out


WARMUP = [("step", 240)]  # tick counts well above the touch windows before anything happens

SCRIPTS = {
    # blue shoots at the orange goal (car 1, passed by car 3), the ball flies in: shot, then goal
    "shot_then_goal": (True, [("ball", (0.0, 2500.0, 300.0), (0.0, 2500.0, 0.0)), ("hit", 3, 100), ("hit", 1, 35),
                              ("step", 1), ("update",)] + _ticks(70, 2)),
    # shot too soon after the touch (inside shotTouchMinDelay), then one in time
    "touch_delay": (True, [("ball", (500.0, 2000.0, 200.0), (-100.0, 2600.0, 100.0)), ("hit", 1, 10),
                           ("step", 1), ("update",), ("hit", 1, 35), ("step", 1), ("update",)] + _ticks(6, 3)),
    # shot, then orange car 2 in the ball's path knocks it back: save
    "save": (True, [("car", 2, (0.0, 3500.0, 17.0)), ("ball", (0.0, 1500.0, 130.0), (0.0, 2500.0, 0.0)),
                    ("hit", 1, 35), ("step", 1), ("update",)] + _ticks(60, 2)),
    # the same with state-set detection off and a ball state set midway (the tick gap wraps: no save)
    "save_no_detection": (False, [("ball", (0.0, 2500.0, 300.0), (0.0, 2500.0, 0.0)), ("hit", 1, 35), ("step", 1),
                                  ("update",), ("step", 3), ("update",),
                                  ("ball", (0.0, 3200.0, 300.0), (0.0, -1500.0, 200.0)), ("hit", 2, 0),
                                  ("step", 1), ("update",)] + _ticks(4, 2)),
    # slow ball (below shotMinSpeed), then a state set with detection on (persistent info reset), then a shot
    # at the blue goal by orange
    "slow_and_reset": (True, [("ball", (0.0, -2500.0, 300.0), (0.0, -1200.0, 0.0)), ("hit", 2, 40), ("step", 1),
                              ("update",), ("step", 2), ("update",),
                              ("ball", (100.0, -2600.0, 300.0), (0.0, -2600.0, 50.0)), ("hit", 4, 200), ("hit", 2, 35),
                              ("step", 1), ("update",)] + _ticks(40, 3) + [("reset",), ("step", 1), ("update",)]),
}

SCRIPTS = {k: (auto, WARMUP + ops) for k, (auto, ops) in SCRIPTS.items()}
