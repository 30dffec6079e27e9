"""Known-answer checks of the oracle's fp64 triangle/box test
(src/symvox/test_triangle_box.cpp): inclusive contact, separating axes."""
import numpy as np

import oracle_py


def tri(*v):
    return np.array(v, np.float32)


def test_triangle_through_box():
    assert oracle_py.tri_box((0, 0, 0), 1.0, tri(-2, 0, 0, 2, 0.5, 0, 0, -2, 0.1))


def test_far_triangle():
    assert not oracle_py.tri_box((0, 0, 0), 1.0, tri(5, 5, 5, 6, 5, 5, 5, 6, 5))


def test_face_contact_is_inclusive():
    # triangle lying in the plane x = 1 touches the box [-1,1]^3
    assert oracle_py.tri_box((0, 0, 0), 1.0, tri(1, -0.5, -0.5, 1, 0.5, -0.5, 1, 0, 0.5))


def test_just_outside_face():
    assert not oracle_py.tri_box((0, 0, 0), 1.0, tri(1.001, -0.5, -0.5, 1.001, 0.5, -0.5, 1.001, 0, 0.5))


def test_edge_axis_separation():
    # bounding boxes overlap but an edge cross-product axis separates
    assert not oracle_py.tri_box((0, 0, 0), 0.5, tri(0.9, 0.9, -1, 1.0, 0.4, -1, 0.4, 1.0, 1))


def test_plane_test():
    # plane of the triangle passes beside the box corner
    assert not oracle_py.tri_box((0, 0, 0), 0.25, tri(0.8, 0, 0, 0, 0.8, 0, 0, 0, 0.8))
    assert oracle_py.tri_box((0, 0, 0), 0.25, tri(0.7, 0, 0, 0, 0.7, 0, 0, 0, 0.7))
