"""CPU oracle for flowMC's sampling hot path -- TEST INFRASTRUCTURE ONLY.

A float64 NumPy restatement of the reference algorithms (flowMC v0.4.5),
each function citing the reference file:line it follows. Every random draw
is an explicit input array, so the CUDA path and the oracle consume the same
normals and uniforms.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only to check results against it (or as
the timed CPU baseline); the product path (``flowmc_gb300``) never does.

Pinning: the reference's own tests hold no numeric golden vectors, only
known-answer/statistical pins (acceptance -> 1 at tiny steps, N(0, I)
moments, leapfrog reversibility, determinism, shapes); the oracle is checked
against all of them in ``tests/test_oracle.py``, and its gradients against
central finite differences. In addition ``tests/golden/make_golden.py`` runs
the reference's own MALA, HMC and GaussianRandomWalk kernels and its
RQSpline (knots, forward, inverse) on scripted normals and uniforms, with
small stand-ins for the JAX API (JAX itself is not installed), and
``tests/test_golden.py`` requires the oracle to reproduce those outputs in
float64. JAX's threefry key streams, Equinox's Linear init and optax's AdamW
are third-party code absent from the reference tree: the oracle restates
them from their published definitions (parity on RNG streams is therefore
not claimed; explicit noise replaces it).
"""
