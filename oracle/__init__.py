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
* ``ref``      -- runs the reference's own code compiled from its sources by ``Makefile`` (only
  where the reference sources exist): ``_ref/ref_indices`` (its index planner and test-input
  generator) and ``_ref/libref_pipeline.so`` (its host transform path, src/execution/
  execution_host.cpp and what it calls, with FFTW 3 -- absent here -- replaced by the FFTW-API
  shim ``fftw_shim/``, a DFT written for this project).

Parity pinning: index/layout results are pinned bit-exactly against ``_ref`` (fixtures under
tests/golden/). Floating-point results are pinned against the reference's own host transform path
(``ref_pipeline.npz``, produced by ``libref_pipeline.so`` on the inputs of the reference's local
test suite) and against the dense DFT definition, the check the reference's own tests make.
"""
