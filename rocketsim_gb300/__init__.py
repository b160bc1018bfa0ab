"""GB300-native batched RocketSim arena tick.

The simulation runs in the CUDA library built from ``rocketsim_gb300/csrc``
(``rocketsim_gb300/_lib/librsg_gb300.so``) behind the C ABI of
``include/rocketsim_gb300.h``; this package is the Python host side over that
ABI.  Importing it does not touch the GPU; creating an ``ArenaBatch`` does.
"""
from .abi import (ArenaConfig, BallState, BoostPadConfig, CarConfig, CarControls, CarState, MutatorConfig,  # noqa: F401
                  PadState, RSGError, Vec3, RotMat,
                  GAMEMODE_SOCCAR, GAMEMODE_THE_VOID, TEAM_BLUE, TEAM_ORANGE, CAR_OCTANE, CAR_DOMINUS,
                  CAR_PLANK, CAR_BREAKOUT, CAR_HYBRID, CAR_MERC)
from .arena import (Arena, ArenaBatch, Ball, BallPredTracker, Car, GameEventTracker, arena_config, car_config, default_mutator_config, init,  # noqa: F401
                    init_from_mem,
                    CAR_STATE_DTYPE, BALL_STATE_DTYPE, PAD_STATE_DTYPE, CONTROLS_DTYPE)
from .arena_mesh import arena_cmf, build_arena_mesh  # noqa: F401
