"""GB300-native BAMF hot path: the cRJMCMC reversible-jump sampler and the
findROI / gaussMLE front end, as CUDA kernels for sm_103a behind a C ABI
(include/bamf.h, libbamf_gb300.so)."""
__version__ = "0.1.0"
