"""CPU reference of the search driver (test infrastructure): depth-first
branch and prune with the oracle's Gauss-Seidel fixpoint at every node and the
same branching rule as pir_search (bisect the first unfixed decision variable,
or the one with the smallest domain; lower half first)."""
import numpy as np


def cpu_search(oracle, op, x, y, z, store, dec, order=0, max_solutions=0, max_nodes=0):
    """op/x/y/z: installed bytecode; store: the base store (nvars x 2).  Returns
    (solutions in depth-first order, nodes propagated, failures)."""
    dec = np.asarray(dec)
    stack = [np.array(store, np.int32, copy=True)]
    sols, nodes, fails = [], 0, 0
    while stack:
        if max_nodes and nodes >= max_nodes:
            break
        s = np.ascontiguousarray(stack.pop())
        nodes += 1
        rc, _ = oracle.fixpoint(op, x, y, z, s)
        if rc == oracle.FAILED:
            fails += 1
            continue
        l, u = s[dec, 0], s[dec, 1]
        free = np.where(l < u)[0]
        if len(free) == 0:
            sols.append(l.copy())
            if max_solutions and len(sols) >= max_solutions:
                break
            continue
        k = free[0] if order == 0 else free[np.argmin((u[free].astype(np.int64) - l[free]))]
        v = dec[k]
        lo, hi = int(s[v, 0]), int(s[v, 1])
        mid = lo + (hi - lo) // 2
        right = s.copy()
        right[v] = (mid + 1, hi)
        left = s.copy()
        left[v] = (lo, mid)
        stack.append(right)
        stack.append(left)
    return sols, nodes, fails
