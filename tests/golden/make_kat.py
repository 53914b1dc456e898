"""Writes kat.json: known answers for the reference's own fixtures.

The reference has no golden outputs for the step.  Its bench fixtures come
without expected values, so the answers below were derived by hand from the
reference source, step by step, and are written here as literals (nothing is
computed by the oracle or the GPU code):

K1  solveConstraint testConstraint testObjPair
    (shapes/bench/Physics/Constraint/Benchmark.hs:11-35; Constraint.hs:164-221):
    n = (0,1), xa = (0,0), xb = (0,4), p = (0,2) give
    J = (-0, -1, 0 | 0, 1, 0), b = 0.  v = (1,1,0 | 1,-1,0), InvMass2 (1,2) each:
    J.v = -2, (J*M^-1).J = 2, lambda = -(-2 + 0)/2 = 1, so both bodies end with
    velocity (1, 0) and rotational velocity 0.
K2  OS.contact testOptBoxes (shapes/bench/Physics/Contact/Benchmark.hs:16-30):
    A = box (0,0) 4x4, B = box (1,3) 2x2 (rectangleVertices, CCW from (+w/2,+h/2)).
    minOverlap A B: edge 0 normal (0,1), depth 2 - 2 = 0 (first strict minimum).
    minOverlap B A: edge 2 normal (0,-1), depth -2 - (-2) = 0.  0 < 0 is false,
    so the result is Flip with B's edge 2 penetrated by A's vertex 0 (2,2).
    penetratingEdge picks (A0, A1) since |(A1-A0).n| = 0 < |(A0-A3).n| = 4.
    Clip 1 (perpLine2 (0,2) (2,2)) clips the right end to (0,2); clip 2 keeps both;
    clip 3 intersects parallel lines: det = -0, 1/det = -inf, the point is NaN,
    every comparison is false, nothing is clipped.  flattenContactPoints orders by
    descending vertex index and Flip swaps the feature keys:
      ((1,2), Flip (n=(0,-1), p=(0,2), d=0)), ((0,2), Flip (n=(0,-1), p=(2,2), d=0)).
K3  length (unorderedPairs n) == n(n-1)/2 for n in [0, 30]
    (shapes/test/Physics/Broadphase/AabbSpec.hs:8-16).
"""
import json
from pathlib import Path

KAT = {
    "K1": {
        "j": [-0.0, -1.0, 0.0, 0.0, 1.0, 0.0],
        "b": 0.0,
        "a": [1.0, 1.0, 0.0, 1.0, 2.0],
        "b_obj": [1.0, -1.0, 0.0, 1.0, 2.0],
        "a_after": [1.0, 0.0, 0.0],
        "b_after": [1.0, 0.0, 0.0],
    },
    "K2": {
        "a": {"center": [0.0, 0.0], "size": [4.0, 4.0]},
        "b": {"center": [1.0, 3.0], "size": [2.0, 2.0]},
        "contacts": [
            {"features": [1, 2], "flip": 1, "normal": [0.0, -1.0], "point": [0.0, 2.0], "depth": 0.0},
            {"features": [0, 2], "flip": 1, "normal": [0.0, -1.0], "point": [2.0, 2.0], "depth": 0.0},
        ],
    },
    "K3": {"n_max": 30},
}

if __name__ == "__main__":
    out = Path(__file__).resolve().parent / "kat.json"
    out.write_text(json.dumps(KAT, indent=1) + "\n")
    print(out)
