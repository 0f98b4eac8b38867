"""Host-side helpers of the measurement path (sources/math_utils.py).

Unit constants, coordinate transforms, the indefinite Simpson integral used
for dwell times and transfer probabilities, and the free-packet predictions.
"""
from __future__ import annotations

import math

import numpy as np

planck_constant = 2.0 * math.pi          # sources/math_utils.py:3-6
reduced_planck_constant = 1.0
electron_rest_mass = 1.0


def transform_center_origin_to_corner_origin_system(pos, box_dimensions):
    return np.asarray(pos) + np.asarray(box_dimensions) * 0.5


def transform_corner_origin_to_center_origin_system(pos, box_dimensions):
    return np.asarray(pos) - np.asarray(box_dimensions) * 0.5


def normalize(v):
    v = np.asarray(v, dtype=np.float64)
    return v / math.sqrt(float(np.dot(v, v)))


def classical_momentum(mass, velocity):
    return mass * np.asarray(velocity, dtype=np.float64)


def get_de_broglie_wave_length_bohr_radii(momentum):
    if momentum == 0.0:
        return math.inf
    return planck_constant / momentum


def cut_bounding_box(arr, bottom, top):
    return arr[bottom[0]:top[0], bottom[1]:top[1], bottom[2]:top[2]]


def nearest_power_of_2(n: int) -> int:
    a = int(math.log2(n))
    return n if 2 ** a == n else 2 ** (a + 1)


def indefinite_simpson_integral(array, dt):
    """sources/math_utils.py:199-234: running Simpson integral, trapezoid for the first interval."""
    array = np.asarray(array)
    n = array.size
    if n == 0:
        return np.empty(0, dtype=array.dtype)
    if n == 1:
        return np.array([0.0], dtype=array.dtype)
    if n == 2:
        return np.array([0.0, (array[0] + array[1]) / 2.0], dtype=array.dtype)
    is_even = n % 2 == 0
    odd_section = n - 1 if is_even else n
    even_section = n if is_even else n - 1
    integral = np.zeros(n, dtype=np.float64)
    integral[1] = 3.0 * (array[0] + array[1]) / 2.0
    for i in range(2, odd_section, 2):
        integral[i] = integral[i - 2] + array[i - 2] + 4.0 * array[i - 1] + array[i]
    for i in range(3, even_section, 2):
        integral[i] = integral[i - 2] + array[i - 2] + 4.0 * array[i - 1] + array[i]
    return integral * dt / 3.0


def predict_free_space_standard_devation(delta_t, sigma0, mass, step_count):
    """sources/math_utils.py:237-251."""
    a = sigma0 * 2.0
    t = np.arange(step_count, dtype=np.float64) * delta_t
    return np.sqrt(a ** 2 + 4.0 * (1.0 / mass ** 2) * t ** 2 / a ** 2) / 2.0


def predict_free_space_expected_location(delta_t, x0, velocity, step_count):
    """sources/math_utils.py:254-267."""
    return x0 + np.arange(step_count, dtype=np.float64) * delta_t * velocity
