"""Drop-in subset of the reference's ``phitest`` package: the render + advect hot
path (``phitest.render``) backed by the GB300 CUDA library ``libgft.so``."""
