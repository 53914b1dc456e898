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
K4  Circle.contact (Circle (-1,0) 1.1) (Circle (1,0) 1.1)
    (shapes/bench/Physics/Contact/Circle/Benchmark.hs:8-11; Contact/Circle.hs:27-56):
    ab = (2, 0), rab = 1.1 + 1.1 = 2.2000000000000002, rab^2 = 4.840000000000001 >= 4,
    |ab| = 2, n = (1, 0); a' = 1.1 n + (-1, 0) = (0.10000000000000009, 0),
    b' = -1.1 n + (1, 0) = (-0.10000000000000009, 0) (the y sum -0 + 0 is +0), so the
    centre is ((a' + b') / 2) = (0, 0) and the depth 2.2000000000000002 - 2 =
    0.20000000000000018.  Keyed (0, 0), Same (Contact.hs:25-29).
K5  GJK.closestSimplex (makeOptBox 0 0 1.9 1.9) p for the three points of
    shapes/bench/Physics/Contact/GJK/Benchmark.hs:10-17, each taken through
    CircleVsHull.generateContacts with a circle of radius 0.1 centred on p (the
    circle penetrates; Contact.hs:30-34 keys it (0, hull feature), Same).  The box's
    vertices are (+-0.95, +-0.95) counter-clockwise from (0.95, 0.95) (1.9 / 2 =
    0.95).  support returns the first vertex of largest projection (ConvexHull.hs:124-128).
    p = (1, 1): d = p - v0 = (0.05.., 0.05..), support v0 = the simplex's own vertex, so
      the search stops at Simplex1 v0: the point v0, b = p - v0, |b| = sqrt(2) 0.05.. ,
      normal -(b/|b|) = (-0.7071067811865475, -0.7071067811865475), depth 0.1 - |b| =
      0.029289321881345184, feature 0.
    p = (0, 1): d = (-0.95, 0.05..), support v1; Simplex2 (v1, v0); ab = (1.9, 0) and
      ao = (0.95, 0.05..) point the same way, next d = (ab x ao) x ab = (-0, 0.18..);
      support v0 (v1 ties, not strictly larger): a repeat, the search stops at
      Simplex2 (v1, v0).  closestAlong: a = v1, u = (1, 0), t = 0.95, point (0, 0.95);
      b = (0, 0.05..), normal (-0, -1), depth 0.1 - 0.05.. = 0.04999999999999996, feature 1.
    p = (0, 0.9): d = (-0.95, -0.05..), support v2; Simplex2 (v2, v0), next d points
      to (-, +), support v1; Simplex3 (v1, v2, v0) encloses p (neither abc x ac nor
      ab x abc points toward p): no contact.
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
    "K4": {
        "a": {"center": [-1.0, 0.0], "radius": 1.1},
        "b": {"center": [1.0, 0.0], "radius": 1.1},
        "contact": {"features": [0, 0], "flip": 0, "normal": [1.0, 0.0], "point": [0.0, 0.0],
                    "depth": 0.20000000000000018},
    },
    "K5": {
        "box": {"center": [0.0, 0.0], "size": [1.9, 1.9]},
        "radius": 0.1,
        "cases": [
            {"center": [1.0, 1.0], "contact": {"features": [0, 0], "flip": 0,
                                               "normal": [-0.7071067811865475, -0.7071067811865475],
                                               "point": [0.95, 0.95], "depth": 0.029289321881345184}},
            {"center": [0.0, 1.0], "contact": {"features": [0, 1], "flip": 0, "normal": [-0.0, -1.0],
                                               "point": [0.0, 0.95], "depth": 0.04999999999999996}},
            {"center": [0.0, 0.9], "contact": None},
        ],
    },
}

if __name__ == "__main__":
    out = Path(__file__).resolve().parent / "kat.json"
    out.write_text(json.dumps(KAT, indent=1) + "\n")
    print(out)
