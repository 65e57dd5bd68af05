"""sphugo_gb300 -- GB300-native (sm_103a) implementation of sphugo's 2D SPH step.

The compute path is libsphgpu.so (hand-written CUDA, C ABI in include/sphgpu.h);
this package is its host-side mirror of the reference's Go ``sim`` API.
"""
from .sim import (  # noqa: F401
    ConfigError,
    Ensemble,
    MakeConfig,
    MakeConfigFromFile,
    MakeSimulation,
    MakeSimulationFromConf,
    MakeSimulationFromConfig,
    MakeUniformRectSpawner,
    PointSource,
    Reflections,
    Simulation,
    SphConfig,
    UniformRectSpawner,
    Vec2,
)
