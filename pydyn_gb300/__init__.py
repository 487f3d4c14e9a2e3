"""pydyn_gb300: TM5's dynamic step as pydyn transcribes it, on one GB300 (sm_103a), float64.

The operators of pydyn's dynamic step -- x/y/z slopes advection with Check_CFL sub-cycling on
the reduced grid, convection with Kzz diffusion folded in, CH4 emission and chemistry, and the
zoom tree -- are hand-written CUDA kernels behind a C ABI (include/gbdyn.h), called from
Python through ctypes.  The state stays resident in device memory; the host drives the
operator sequence (pydyn_gb300.zoom, pydyn_gb300.driver) and captures a whole step as a CUDA
graph.  Results are bitwise those of pydyn's NumPy reference.
"""

__version__ = "0.1.0"
