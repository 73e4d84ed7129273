"""speccodelib_gb300 -- GB300-native pseudo-spectral Navier-Stokes step.

The product is ``lib/libspecns.so`` (hand-written sm_103a CUDA behind the C
ABI of ``include/specns.h``); this package builds it (`build`) and mirrors the
reference's subroutine interface over it (`specns`).
"""
from .specns import (SC_FP32, SC_FP64, SC_SGS_DYNSMAG, SC_SGS_NONE, SC_SGS_SMAG,  # noqa: F401
                     SC_MASK_AFTER_STEP, SC_MASK_RHS_AND_STEP, SpecNSError, SpectralNS,
                     convec_dns, dealiasing, default_params, dynsmag, force, projection,
                     smag, symmetrize, Ensemble2D, force_rot, convecphi_dns,
                     skewness, enstrophy, ab2v_dt, forcephi, forcephi_rot, hermitianize,
                     fp64_peak_probe)
