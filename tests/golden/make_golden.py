"""Generates tests/golden/c1_small.npz from the CPU oracle.

The reference (Julia + Mantis.jl) cannot run on this machine, so these vectors
pin the oracle against itself across machines (x86 build host, Arm GPU host)
and across edits; the reference pins are the known-answer tests and method
identities in test_oracle.py. Inputs: 512 markers of the 16x16 [-6,6]^2
configuration (anisotropic Gaussian, sigma = (1, 0.5), numpy seed 1234) and the
3-marker compute_moments case of the reference's main_helpers.jl:28-38.

Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402


def main():
    bp = np.linspace(-6.0, 6.0, 17)
    rng = np.random.default_rng(1234)
    N = 512
    v = np.asfortranarray(np.column_stack([rng.standard_normal(N), 0.5 * rng.standard_normal(N)]))
    w = np.full(N, 1.0 / N)
    om = oracle.OracleMesh(bp, bp, 6)
    f = om.l2_project(v, w)
    r = om.compute_r(f)
    S = om.entropy(f)
    G = om.compute_G(v, om.mass_solve(r))
    dotv = om.collision(v, w, G)
    mv = np.array([[1.0, 2.0], [-3.0, 0.5], [0.0, -1.0]])
    mw = np.array([0.2, 0.3, 0.5])
    mo = np.array(oracle.moments(mv, mw))
    np.savez_compressed(os.path.join(HERE, "c1_small.npz"), bp=bp, v=v, w=w, f=f, r=r, S=S, G=G,
                        dotv=dotv, mom_v=mv, mom_w=mw, mom_out=mo)
    print("wrote c1_small.npz")


if __name__ == "__main__":
    main()
