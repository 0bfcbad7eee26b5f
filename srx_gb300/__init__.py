"""GB300-native EVP-FFT equilibrium iteration for SRX-format RVEs.

The compute path is the CUDA library built from ``srx_gb300/csrc`` and
exposed through the C ABI in ``include/evpg.h``; this package holds the
ctypes binding, the host-side job driver and the input-format helpers.
"""
