"""CPU oracle for pmwd's particle-mesh path -- TEST INFRASTRUCTURE ONLY.

This package is a NumPy/SciPy restatement of the reference algorithms
(pmwd ``pm_util.py``, ``scatter.py``, ``gather.py``, ``gravity.py``,
``nbody.py``, ``cosmology.py``, ``boltzmann.py``, ``lpt.py``, ``modes.py``,
``spec_util.py``).  Each function cites the reference ``file:line`` it follows.

It exists to check the CUDA path.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it.  The product package
``pmwd_gb300`` never imports it, and the product path never falls back to it.

Parity pinning: the reference is JAX code and JAX is not importable where
this oracle was written, so it could not be run to produce golden vectors.
The oracle is pinned by (i) the known-answer properties of the reference's
own test file ``tests/pm_test.py`` (centred-particle scatter, scatter sum,
uniform gather, reversibility), (ii) adjoint checks against autograd of an
independent float64 torch restatement (``oracle.ad``), (iii) the
white-noise draw restated from JAX's published algorithm (``oracle.prng``,
checked against the Random123 known answers and JAX's documented draws), so
that a seed gives pmwd's own realisation, and (iv) through it, outputs pmwd
published for seeded runs (``tests/golden/published_pmwd.json``: the
quickstart notebook's statistics and cosmology gradients, the adjoint
paper's 64 repeated gradient runs), which the GPU path reproduces.
"""
