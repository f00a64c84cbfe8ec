"""Oracle chains as plain functions, for process pools in the tests.

TEST INFRASTRUCTURE ONLY: the GPU tests compare the device chains of the
benchmark workload with these oracle runs; a spawned process pool runs one
chain per call (the oracle is single threaded).
"""
from __future__ import annotations

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def chain_moves(args):
    """One oracle chain: pre-loading with `create` molecules from `seed`,
    then `moves` main-loop moves.  Returns (coordinates after pre-loading,
    per-move records, energy before each displacement-type move of the
    moving molecule).  The record tuples are (move, iguest, choice,
    overlap, accepted, estep, rande, nmols_after)."""
    d, seed, create, moves = args
    import numpy as np
    from oracle.binding import Oracle
    o = Oracle(d)
    o.seed(seed)
    if create:
        o.create_molecules(1, create)
    mol = o.locguest(1)
    xyz0 = np.array(o.coords(mol))
    recs, e_old = [], []
    for _ in range(moves):
        # the moving molecule's energy before the move (its deletion energy)
        # is needed only for displacement-type moves, whose choice is known
        # after the move: run the move on a saved copy first
        o.save_state()
        r = o.run(1)[0]
        if r.move in (3, 4, 5, 6) and r.choice >= 1:
            o.restore_state()
            e = o.deletion_energy(1, r.choice)["estep"]
            o.restore_state()
            r = o.run(1)[0]
        else:
            e = 0.0
        recs.append((r.move, r.iguest, r.choice, r.overlap, r.accepted, r.estep, r.rande,
                     r.nmols_after))
        e_old.append(e)
    return xyz0, recs, e_old
