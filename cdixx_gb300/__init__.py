"""GB300-native CDI phase-retrieval path (FFT, modulus projection, HIO/RAAR/ER
updates, shrinkwrap) behind a C ABI (include/cdx.h).  Python modules here are
bindings and host utilities; the computation is in ``_lib/libcdx.so``."""
__version__ = "0.1.0"
