"""CPU oracle for the quantax VMC inner loop.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline arm may import this package, and only as the checker or the timed CPU
restatement.  The product package (quantax_gb300) never imports it and has no CPU
fallback.

Parity status: the reference (pure JAX/Equinox) cannot be imported where this was built,
so the oracle is a restatement of the reference's algorithms with file:line citations.
It is pinned against the reference's own known answers: the exact-diagonalisation
energies printed in tutorials/J1J2.ipynb (4x4 Heisenberg with Marshall sign rule
-44.91393283371544, 4x4 J1-J2 J2=0.5 -33.831693405579394), against the published
Philox4x32-10 known-answer vectors, and against the reference's own self-consistency
asserts (local-update psi == direct psi, local-update E_loc == direct E_loc,
tutorials/local_updates.ipynb).  There are no fixed-seed golden psi / E_loc / O / step
vectors in the reference; those values are pinned only through the restated algorithm.
"""
