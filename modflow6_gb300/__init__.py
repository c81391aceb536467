"""GB300-native Iterative Model Solution (IMS) hot path for MODFLOW 6.

The compute lives in libgbims.so (C ABI: include/gbims.h); this package holds
the host-side mirror of the IMS interface (ims.py), DIS grid models (dis.py),
the device-resident solution (solution.py) and the build helper (build.py).
"""
__version__ = "0.1.0"
