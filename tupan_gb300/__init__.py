"""tupan_gb300: GB300-native (sm_103a) backend for Tupan's pairwise gravity kernels.

    from tupan_gb300.lib import extensions
    extensions.acc.calc(ips, jps)          # like tupan.lib.extensions

The compute path is libtupan_gb300.so (tupan_gb300/csrc, C ABI in
include/tupan_gb300.h); build it with `python -m tupan_gb300.build`.
"""
__version__ = "0.1.0"
