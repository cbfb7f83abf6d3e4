"""gravitation_gb300 -- GB300-native all-pairs n-body engine for the gravitation
benchmark suite's plugin API.

  engine.Engine      FP64 state + persistent stage-1 / FP64 stage-2 launches (C ABI)
  plugin.GB300Stages universe_base hooks; kernel/gb1 is the drop-in kernel package
  tune.Tuner         tile-shape autotuner with a JSON cache
  scenarios          seeded workloads
  build              nvcc build of libgravgb300.so (sm_103a)
"""

__version__ = '0.1.0'
