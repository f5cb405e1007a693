"""CPU oracle for the fluidLB D2Q9 time step.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` use it, and only as the checker or as the timed CPU baseline.

Contents
--------
``lbm_np``      FP64 NumPy restatement of the reference's CPU kernels, in the
                reference's own padded AoS ``[node][q]`` layout and operation
                order (bit-exact with the reference kernels run as Python).
``setup``       builds the reference-layout state (ghost ring, boundary node
                lists, circle solids, initial fields) from ``simulation.py``
                style case dictionaries.
``lbm_oracle.c`` the same restatement in C (OpenMP over nodes), used for
                large cases and as the timed CPU baseline; ``clib`` loads it.

Parity pinning: the reference has no tests, golden files or known-answer
vectors for this path.  The restatement is pinned against fixtures produced by
running the reference's own ``pylabolt/parallel/cpu/*.py`` kernels (with a
stand-in ``numba`` module that turns ``njit`` into the identity and
``prange`` into ``range``); the generating script is
``tests/golden/make_golden.py`` and the fixtures are ``tests/golden/*.npz``.
"""
