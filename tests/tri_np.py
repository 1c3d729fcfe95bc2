"""Moller-Trumbore of AccelerationStructure.h:70-97 in numpy float32 (no fused
multiply-add), used by tests to confirm tie cases."""
import numpy as np

f = np.float32


def intersect_t(ray, tri):
    o = ray[0:3].astype(f)
    d = ray[3:6].astype(f)
    A, B, C = (tri[0:3].astype(f), tri[3:6].astype(f), tri[6:9].astype(f))
    E1 = B - A
    E2 = C - A
    P = np.array([d[1] * E2[2] - d[2] * E2[1], d[2] * E2[0] - d[0] * E2[2], d[0] * E2[1] - d[1] * E2[0]], f)
    det = f(f(E1[0] * P[0] + E1[1] * P[1]) + E1[2] * P[2])
    det = f(f(1.0) / det)
    T = o - A
    Q = np.array([T[1] * E1[2] - T[2] * E1[1], T[2] * E1[0] - T[0] * E1[2], T[0] * E1[1] - T[1] * E1[0]], f)
    t = f(f(f(E2[0] * Q[0] + E2[1] * Q[1]) + E2[2] * Q[2]) * det)
    return t
