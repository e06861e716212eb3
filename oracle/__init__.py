"""CPU oracle for the GB300 SpFFT library -- TEST INFRASTRUCTURE ONLY.

Nothing in the library imports this package. Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` use it, and only to produce expected results or as the timed CPU baseline.

* ``indices``  -- numpy restatement of the reference's index conversion
  (src/compression/indices.hpp:120-186, src/parameters/parameters.cpp:143-180).
* ``pipeline`` -- numpy/scipy restatement of the reference's host execution engine
  (src/execution/execution_host.cpp:49-352 with compression_host.hpp, symmetry_host.hpp,
  transpose_host.hpp and the pruned y transform of transform_1d_host.hpp:154-231); FFTW calls are
  replaced by scipy.fft (pocketfft) transforms of the same direction and normalisation.
* ``dense``    -- the dense 3D DFT oracle of the reference's tests
  (tests/test_util/test_transform.hpp:33-276).
* ``ref``      -- runs ``_ref/ref_indices``, the reference's own index code compiled from its
  sources by ``Makefile`` (only where the reference sources exist).

Parity pinning: index/layout results are pinned bit-exactly against ``_ref`` (fixtures under
tests/golden/). Floating-point results are pinned against the dense DFT definition, which is the
check the reference's own tests make; the reference ships no floating-point golden vectors and its
FFT library (FFTW 3) is not available here.
"""
