"""CPU oracle for the CMM-on-the-sphere hot path.

TEST INFRASTRUCTURE ONLY.  This package restates, in numpy/scipy, the
algorithms of the reference ``cmm_s2/core`` modules that the GPU library
replaces.  It exists to check the GPU library and to time a CPU baseline:
only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it.  The GPU library never calls it and has no CPU
fallback.

Pinning: ``tests/golden/make_golden.py`` runs the reference's own code
(imported with small import shims) on frozen inputs and stores its outputs
in ``tests/golden/*.npz``; ``tests/test_oracle_golden.py`` checks this
package against those files.  The MWSS spherical-harmonic transform of the
third-party ``pyssht`` package (ssht + ducc0, version unpinned by the
reference) is absent, so ``oracle.sht`` restates the published MWSS sampling
theorem; it is pinned only on band-limited closed-form fields (the
reference's Rossby-Haurwitz and Poisson test pairs).
"""
