"""qsf_gb300 -- GB300 (sm_103a) split-operator step for QSF's reduced-dimensionality TDSE.

The compute path is libqsfgpu.so (hand-written CUDA, C ABI in include/qsf_gpu.h);
this package holds its Python binding and a host-side mirror of the reference's
propagator / field / coupling vocabulary.  There is no CPU fallback: importing the
grid classes requires the built library.
"""
from ._lib import QsfError, lib  # noqa: F401
from .grid import (ABS_CAP, ABS_COS8, BORDERS, Batch, Grid, MODE_IM, MODE_RE, OBS_EKIN, OBS_EPOT, OBS_FLUX, OBS_NORM, OP_IDENTITY,  # noqa: F401
                   OP_KINETIC, OP_POTENTIAL, POT_COULOMB, POT_EBERLY, POT_ECKHARDT_SACHA, POT_NONE, REP_P, REP_X,
                   ZOA_FLUX_2D, ZOA_FLUX_2D_SIMPLE, ZOA_FLUX_3D, fft_radices)
from .physics import (AXIS_X, AXIS_Y, AXIS_Z, GAUGE_LENGTH, GAUGE_VELOCITY, PULSE_CHEMPHYS, PULSE_CONST,  # noqa: F401
                      PULSE_SIN, PULSE_SIN2_SIN, Coupling, Field, Pulse, field_from_intensity, omega_from_wavelength)
from .propagator import SplitPropagator  # noqa: F401
