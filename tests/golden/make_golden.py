"""Regenerates tests/golden/oracle_golden.npz: FP64 oracle outputs on small
seeded slices of the benchmark workloads (verdicts, edge first-hit indices,
forward kinematics).  The reference's own FP64 code (KrisLibrary) cannot be
built or imported here, so these vectors come from the oracle, whose
conventions are pinned by tests/test_oracle.py (known answers, the rotation
vector of the reference's tests/test_math_so3.py, brute-force checks).

Usage: python tests/golden/make_golden.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from klampt_gb300 import scenes as sc  # noqa: E402
from oracle import oracle_py as op  # noqa: E402


def main():
    out = {}
    robot, env, q = sc.scene_cfg0()
    o = op.Oracle(robot, env)
    q0 = q[:256]
    eh, sh, _ = o.check_configs(q0, nthreads=os.cpu_count() or 2)
    out.update(cfg0_q=q0, cfg0_env=eh, cfg0_self=sh)
    robot1, env1, (qa, qb, ns) = sc.scene_cfg1()
    o1 = op.Oracle(robot1, env1)
    sel = slice(0, 256)
    fh, _ = o1.check_edges(qa[sel], qb[sel], ns[sel], nthreads=os.cpu_count() or 2)
    out.update(cfg1_qa=qa[sel], cfg1_qb=qb[sel], cfg1_ns=ns[sel], cfg1_first_hit=fh)
    qf = sc.uniform_configs(robot1, 16, np.random.default_rng(77))
    out.update(fk_q=qf, fk_T=np.stack([o1.fk(x.astype(np.float64)) for x in qf]))
    np.savez_compressed(os.path.join(HERE, "oracle_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "oracle_golden.npz"))


if __name__ == "__main__":
    main()
