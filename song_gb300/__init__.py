"""GB300 second-order perturbation evolver (SONG perturbations2.c hot path).

The product is the C ABI in include/song2.h, implemented by
song_gb300/csrc (host C + sm_103a CUDA) and built in-tree by
song_gb300.build.build() into song_gb300/_build/libsong2.so.  capi.py is the
ctypes binding; problem.py sets up specs and tables for Python callers.
"""
