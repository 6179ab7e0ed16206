"""kylin_v_gb300: GB300-native Holstein TDVP hot path (Kylin-V compatible).

The compute path lives in the CUDA/C++ library ``libkvgpu.so`` (built from
``csrc/``) behind the C ABI declared in ``include/kvgpu.h``; this package holds
the host-side mirror of the reference's operator surface, the workload
generators and the file formats.
"""
