"""The CUDA SpMV and row sums visit a row's entries in the order given by a
two-comparison rule (device.cuh, row_ordered) instead of sorting columns.
Check on the CPU that the rule reproduces ascending column order for every
row of the four systems on several geometries, using the oracle's patterns."""
import numpy as np
import pytest

from helpers import params, solver
from ns3d_gb300 import capi, synth

# slot names in nbr order W,E,S,N,B,T
W, E, S, N, B, T = range(6)


def rule_order(row, nb):
    out = []
    if nb[W] >= 0 and nb[W] == row - 1:
        out += [nb[S], nb[B], nb[W]]
    else:
        out += [nb[W], nb[S], nb[B]]
    out.append(row)
    if nb[E] >= 0 and nb[E] == row + 1:
        out += [nb[E], nb[T], nb[N]]
    else:
        out += [nb[T], nb[N], nb[E]]
    return [c for c in out if c >= 0]


@pytest.mark.parametrize("shape,frac,seed,direction,border", [
    ((9, 7, 8), 0.7, 1, 1, 0), ((12, 10, 6), 0.5, 2, 2, 1), ((6, 11, 9), 0.85, 3, 3, 2), ((5, 5, 1), 0.8, 4, 1, 0),
    ((1, 6, 7), 0.9, 5, 1, 0), ((14, 3, 3), 0.9, 6, 1, 0)])
def test_rule_matches_sorted_columns(oracle, shape, frac, seed, direction, border):
    img = synth.random_image(shape, frac, seed)
    s = solver(oracle, img, params(oracle, direction=direction, border=border))
    s.assemble_momentum()
    s.assemble_pressure_correction(True)
    for sys in (capi.SYS_U, capi.SYS_V, capi.SYS_W, capi.SYS_P):
        n = s.n(sys)
        if n == 0:
            continue
        _, nbr, _, _ = s.system(sys)
        for r in range(n):
            nb = [int(nbr[d, r]) for d in range(6)]
            got = rule_order(r, nb)
            assert got == sorted(got), (sys, r, nb)
            assert len(got) == 1 + sum(c >= 0 for c in nb)
