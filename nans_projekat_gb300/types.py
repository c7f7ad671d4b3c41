"""Host-side record types of the reference step, as numpy structured dtypes.

These mirror, field for field and byte for byte, the reference's interchange structs:

* ``cube``         -- code/nans.h:303-319 (244 bytes)
* ``sphere``       -- code/nans.h:321-336 (148 bytes)
* ``contact_pair`` -- code/nans.h:338-372 (96 bytes)
* ``collision_type`` values -- code/nans.h:73-89 (CC=0, CS=1, CF=2, SS=3, SF=4)

glm::mat4 is column major (16 floats, column j at [4j, 4j+4)); glm::vec3 is 3 floats.
The same layouts are declared in C in include/nans_gb300.h.
"""
import numpy as np

CC, CS, CF, SS, SF = 0, 1, 2, 3, 4
PAIR_TYPE_NAMES = {CC: "CC", CS: "CS", CF: "CF", SS: "SS", SF: "SF"}

CUBE_DTYPE = np.dtype([
    ("Model", "<f4", (16,)),
    ("Vertices", "<f4", (8, 3)),
    ("Position", "<f4", (3,)),
    ("V", "<f4", (3,)),
    ("Forces", "<f4", (3,)),
    ("Angles", "<f4", (3,)),
    ("W", "<f4", (3,)),
    ("Torque", "<f4", (3,)),
    ("Size", "<f4"),
    ("Mass", "<f4"),
    ("MOI", "<f4"),
])

SPHERE_DTYPE = np.dtype([
    ("Model", "<f4", (16,)),
    ("Position", "<f4", (3,)),
    ("V", "<f4", (3,)),
    ("Forces", "<f4", (3,)),
    ("Angles", "<f4", (3,)),
    ("W", "<f4", (3,)),
    ("Torque", "<f4", (3,)),
    ("Radius", "<f4"),
    ("Mass", "<f4"),
    ("MOI", "<f4"),
])

PAIR_DTYPE = np.dtype([
    ("Type", "<i4"),
    ("DLNormal", "<f4"),
    ("DLNormalSum", "<f4"),
    ("DLTangent1", "<f4"),
    ("DLTangent1Sum", "<f4"),
    ("DLTangent2", "<f4"),
    ("DLTangent2Sum", "<f4"),
    ("PointA", "<f4", (3,)),
    ("PointB", "<f4", (3,)),
    ("N", "<f4", (3,)),
    ("T1", "<f4", (3,)),
    ("T2", "<f4", (3,)),
    ("IndexA", "<i4"),
    ("IndexB", "<i4"),
])

assert CUBE_DTYPE.itemsize == 244
assert SPHERE_DTYPE.itemsize == 148
assert PAIR_DTYPE.itemsize == 96

IDENTITY16 = np.eye(4, dtype=np.float32).reshape(16)
