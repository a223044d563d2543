"""ppafm_gb300 -- the probe-particle AFM hot path (force-field grids, FIRE relaxation,
Fz -> Δf) as hand-written CUDA for GB300 (sm_103a), behind the call signatures of
ppafm.core, ppafm.common, ppafm.HighLevel, ppafm.fieldFFT and ppafm.ocl.AFMulator.

Modules are imported lazily so that host-only helpers work without a GPU.
"""

__version__ = "0.1.0"
