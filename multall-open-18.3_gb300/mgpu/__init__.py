"""mgpu: host side of the GB300 time-marching library for Multall-open 18.3.

The compute path is the CUDA library libmgpu.so (csrc/), exposed through the
C ABI in include/mgpu.h; this package builds it, binds a case's COMMON data
to it by name and drives it.  mgpu.case and mgpu.common_setup stand in for
the reference's input reader and SETUP, which stay outside the hot path.
"""
