"""vpm_gb300 -- GB300-native UJ step for FLOWVPM.jl particle fields.

The package mirrors the reference's user-facing interface around the UJ hook
(ParticleField, kernels, formulations, SFS/relaxation/viscous schemes, the rVPM
RK3 step) and routes every particle-to-particle evaluation through the C ABI of
libvpm_gb300.so (include/vpm_gb300.h) -- hand-written sm_103a kernels, with no
CPU fallback.
"""
from . import _lib
from ._lib import (FP32COMP, FP64, Context, VPMError, default_context, load)
from .particlefield import (ParticleField, ClassicVPM, ReformulatedVPM, Kernel, cVPM, rVPM,
                            formulation_classic, formulation_default, gaussian, gaussianerf, singular,
                            winckelmans,
                            kernel_default, standard_kernels, const1, const2, const3, const4)
from .timeintegration import (AfterUJ, BeforeUJ, ConstantSFS, CoreSpreading, DynamicSFS, Inviscid,
                              NoSFS, Relaxation, SFS_Cd_twolevel_nobackscatter, SFS_Cs_nobackscatter,
                              clipping_backscatter, correctedpedrizzetti, euler, isSFSenabled, noSFS,
                              norelaxation, pedrizzetti, rbf_conjugategradient, rungekutta3, run_vpm,
                              update_particle_states)
from .uj import UJ_gb300, UJ_gb300_cross, UJ_gb300_mixed, zeta_fmm_gb300, zeta_gb300, zeta_gb300_mixed
from . import rings

__all__ = [n for n in dir() if not n.startswith("_")]
