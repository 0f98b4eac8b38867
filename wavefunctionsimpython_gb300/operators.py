"""Operators module — working restatement of sources/operators.py:9-55.

``init_kinetic_operator`` returns the half-step kinetic operator
exp(-i |k|^2 dt / (4 m)) on the grid (the reference's version refers to
undefined names and has no caller); ``init_potential_operator`` multiplies
``P_potential`` by cexp_i(-dt V) (potential_operator.cu:11-15). Both run on
the GPU through the engine and return host arrays.
"""
from __future__ import annotations

import numpy as np

from ._lib import Engine


def init_kinetic_operator(delta_x_3, delta_time: float, mass: float, shape, double_precision: bool = False):
    n = tuple(int(s) for s in shape)
    extent = tuple(float(delta_x_3[i]) * n[i] for i in range(3))
    eng = Engine(n, extent, double_precision=double_precision)
    try:
        return eng.kinetic_operator(delta_time, mass, fraction=0.25)
    finally:
        eng.close()


def init_potential_operator(P_potential: np.ndarray, V: np.ndarray, delta_time: float, delta_x_3=(1.0, 1.0, 1.0)):
    P = np.asarray(P_potential)
    dbl = P.dtype == np.complex128
    n = P.shape
    eng = Engine(n, tuple(float(delta_x_3[i]) * n[i] for i in range(3)), double_precision=dbl)
    try:
        eng.set_potential(np.asarray(V, dtype=np.complex64))
        return eng.potential_operator(delta_time, P)
    finally:
        eng.close()
