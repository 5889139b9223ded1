"""GB300 (sm_103a) implementation of SCCM's PNAMP projected-kernel stage.

Modules: `basis` (m-scheme basis, Wigner d, mesh), `formats` (SCCM file
formats), `synth` (seeded synthetic inputs), `build` (nvcc build of the CUDA
library), `pnamp` (ctypes host over the C ABI in include/pnamp_gpu.h),
`driver` (pair scheduling and kernel-file output).
"""
__version__ = "0.1.0"
