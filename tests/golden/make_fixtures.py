"""Generates tests/golden/fixpoints_small.npz: the CPU oracle's fixpoints of the
1,000-variable / 3,000-propagator workload (seeds 0-9, planted; seeds 0-2 of
the uniform-index variant, which fail), with a hash of every generated
instance so that generator drift on any host is caught.

    python tests/golden/make_fixtures.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "lala-pc_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

PLANTED = list(range(10))
SPEC = list(range(3))


def instance_hash(inst):
    h = hashlib.sha256()
    for a in (inst.lb, inst.ub, inst.op, inst.x, inst.y, inst.z):
        h.update(np.ascontiguousarray(a, np.int32).tobytes())
    return h.hexdigest()[:16]


def cases():
    import workloads as W
    for s in PLANTED:
        yield "planted%d" % s, W.single_small(s)
    for s in SPEC:
        yield "spec%d" % s, W.single_small(s, variant="spec")


def main():
    from oracle import oracle as O
    out = {}
    for name, inst in cases():
        s = inst.store()
        st, info = O.install_and_fixpoint(inst.op, inst.x, inst.y, inst.z, s)
        out[name + "_store"] = s
        out[name + "_status"] = np.int32(st)
        out[name + "_sweeps"] = np.int64(info["sweeps"])
        out[name + "_hash"] = np.array(instance_hash(inst))
    np.savez_compressed(os.path.join(HERE, "fixpoints_small.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
