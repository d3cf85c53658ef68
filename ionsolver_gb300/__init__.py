"""ionsolver_gb300 -- IonSolver's single-node MHD-LBM timestep on one GB300.

The compute path is libionsolver.so (hand-written sm_103a CUDA kernels plus a
C++ host library behind the C ABI of include/ionsolver.h).  This package is
the Python mirror of the reference's Rust API over that ABI.
"""
from .lbm import (FIELDS, Batch, FieldMode, FloatType, Lbm, LbmConfig, ModelType, RelaxationTime, Units, VelocitySet,
                  codec_roundtrip, kernel_launch_count, read_config, taylor_green_fields, write_config)
from .meshes import annulus, cylinder
from ._native import IonError, LIB_PATH

__all__ = ["Lbm", "LbmConfig", "Units", "ModelType", "VelocitySet", "RelaxationTime", "FloatType", "FieldMode",
           "FIELDS", "IonError", "LIB_PATH", "taylor_green_fields", "codec_roundtrip", "kernel_launch_count",
           "cylinder", "annulus", "read_config", "write_config"]
