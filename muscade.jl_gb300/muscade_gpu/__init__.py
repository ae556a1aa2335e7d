"""muscade_gpu: GB300 assemble-and-solve path for Muscade.jl beam models.

Host-side mirror of the reference's model interface (Model, addnode,
addelement, initialize, element types) over the C-ABI library built from
muscade.jl_gb300/csrc (include/muscade_gpu.h).  There is no CPU
implementation of the device path; calls fail if the library is not built.
"""
from .model import Model, State, Disassembler, MuscadeError  # noqa: F401
from .elements import (  # noqa: F401
    EulerBeam3D, Bar3D, Hold, DofConstraint, DofLoad, BeamCrossSection, AxisymmetricBarCrossSection,
    SingleDofCost, SingleUdof, SingleAcost, QuadraticCost,
)
from .solve import solve, SweepXGPU  # noqa: F401


def build(force: bool = False) -> str:
    """Compile the CUDA library for sm_103a in-tree."""
    from . import _lib
    return _lib.build(force=force)


def device_model(model, dis, device: int = 0):
    from .device import DeviceModel
    return DeviceModel(model, dis, device=device)
