"""A small numpy stand-in for the parts of Taichi that the reference's dem.py
physics methods use, so that those methods can be executed from the
reference's own source on the CPU (taichi itself is not installed).

It is test infrastructure for tests/golden/make_physics_golden.py only.  It
supplies:

* vectors and matrices (`Vector3`, `Vector4`, `DEMMatrix`, `Zero3x3`) as
  float64 numpy arrays of class `Vec`, whose `@` sums each row left to right
  with separately rounded products (Taichi's unrolled small-matrix product
  with no fused multiply-add);
* `ti.Matrix.inverse` as the adjugate divided by the determinant, the closed
  form Taichi uses for 3x3 matrices; `ti.Matrix.diag`;
* `tm.length` (square root of the left-folded sum of squares),
  `tm.normalize` (v / length(v)), `tm.dot`, `tm.cross`, `tm.sign` (-1, 0, +1),
  `tm.min`/`tm.max`, `tm.sqrt`, `tm.log`, `tm.pi`;
* `ti.atomic_add(dst, v)`, adding in place into a record's vector field;
* `ti.static`, `ti.abs`, `ti.ndrange`;
* `Field` (a 1-D or 2-D array of records with the dataclass's fields, zero
  initialised) and `record_type` (a dataclass constructor taking keywords,
  missing fields zero).
"""
from __future__ import annotations

import itertools
import math
from types import SimpleNamespace

import numpy as np


class Vec(np.ndarray):
    """float64 vector / matrix with Taichi's small-matrix product."""

    def __matmul__(self, other):
        return matmul(np.asarray(self), np.asarray(other))

    def __rmatmul__(self, other):
        return matmul(np.asarray(other), np.asarray(self))

    def cross(self, other):
        return cross(self, other)

    def norm(self):
        return length(self)


def vec(xs) -> Vec:
    return np.array(xs, dtype=np.float64).view(Vec)


def matmul(a: np.ndarray, b: np.ndarray) -> Vec:
    if b.ndim == 1:
        out = []
        for r in range(a.shape[0]):
            acc = float(a[r, 0]) * float(b[0])
            for k in range(1, a.shape[1]):
                acc = acc + float(a[r, k]) * float(b[k])
            out.append(acc)
        return vec(out)
    out = np.zeros((a.shape[0], b.shape[1]))
    for r in range(a.shape[0]):
        for c in range(b.shape[1]):
            acc = float(a[r, 0]) * float(b[0, c])
            for k in range(1, a.shape[1]):
                acc = acc + float(a[r, k]) * float(b[k, c])
            out[r, c] = acc
    return out.view(Vec)


def dot(a, b) -> float:
    acc = float(a[0]) * float(b[0])
    for k in range(1, len(a)):
        acc = acc + float(a[k]) * float(b[k])
    return acc


def length(a) -> float:
    return math.sqrt(dot(a, a))


def normalize(a) -> Vec:
    return vec(a) / length(a)


def cross(a, b) -> Vec:
    a0, a1, a2 = (float(x) for x in a)
    b0, b1, b2 = (float(x) for x in b)
    return vec([a1 * b2 - a2 * b1, a2 * b0 - a0 * b2, a0 * b1 - a1 * b0])


def sign(x) -> float:
    x = float(x)
    return float(x >= 0.0) - float(x <= 0.0)


def inverse(m) -> Vec:
    a = np.asarray(m, dtype=np.float64)
    det = (a[0, 0] * (a[1, 1] * a[2, 2] - a[2, 1] * a[1, 2])
           - a[1, 0] * (a[0, 1] * a[2, 2] - a[2, 1] * a[0, 2])
           + a[2, 0] * (a[0, 1] * a[1, 2] - a[1, 1] * a[0, 2]))
    inv_det = 1.0 / det
    out = np.empty((3, 3))
    out[0, 0] = inv_det * (a[1, 1] * a[2, 2] - a[2, 1] * a[1, 2])
    out[1, 0] = inv_det * (a[1, 2] * a[2, 0] - a[1, 0] * a[2, 2])
    out[2, 0] = inv_det * (a[1, 0] * a[2, 1] - a[2, 0] * a[1, 1])
    out[0, 1] = inv_det * (a[2, 1] * a[0, 2] - a[0, 1] * a[2, 2])
    out[1, 1] = inv_det * (a[0, 0] * a[2, 2] - a[2, 0] * a[0, 2])
    out[2, 1] = inv_det * (a[0, 1] * a[2, 0] - a[0, 0] * a[2, 1])
    out[0, 2] = inv_det * (a[0, 1] * a[1, 2] - a[0, 2] * a[1, 1])
    out[1, 2] = inv_det * (a[0, 2] * a[1, 0] - a[0, 0] * a[1, 2])
    out[2, 2] = inv_det * (a[0, 0] * a[1, 1] - a[0, 1] * a[1, 0])
    return out.view(Vec)


def atomic_add(dst, v):
    old = np.array(dst)
    dst += v
    return old


class _Matrix:
    inverse = staticmethod(inverse)

    @staticmethod
    def diag(n, val):
        return (np.eye(n) * float(val)).view(Vec)


ti = SimpleNamespace(
    static=lambda x: x,
    abs=lambda x: abs(float(x)),
    atomic_add=atomic_add,
    ndrange=lambda *ns: itertools.product(*(range(n) for n in ns)),
    Matrix=_Matrix,
    f64=float,
    i32=int,
)

tm = SimpleNamespace(
    normalize=normalize,
    cross=cross,
    dot=dot,
    length=length,
    sign=sign,
    min=lambda a, b: min(float(a), float(b)),
    max=lambda a, b: max(float(a), float(b)),
    sqrt=lambda x: math.sqrt(float(x)),
    log=lambda x: math.log(float(x)),
    pi=math.pi,
)


def Vector3(x, y, z) -> Vec:
    return vec([x, y, z])


def Vector4(w, x, y, z) -> Vec:
    return vec([w, x, y, z])


def DEMMatrix(rows) -> Vec:
    return vec(rows)


def Zero3x3() -> Vec:
    return vec(np.zeros((3, 3)))


# Field shapes of the reference's dataclasses (dem.py:808-893): name -> shape
# (() for a scalar, (3,) for a vector, (3, 3) for a matrix).
GRAIN = {"ID": (), "groupID": (), "materialType": (), "mass": (), "radius": (),
         "contactRadius": (), "position": (3,), "velocity": (3,), "acceleration": (3,),
         "force": (3,), "quaternion": (4,), "omega": (3,), "omega_dot": (3,),
         "inertia": (3, 3), "moment": (3,)}
MATERIAL = {"density": (), "elasticModulus": (), "poissonRatio": ()}
SURFACE = {"coefficientFriction": (), "coefficientRestitution": (),
           "coefficientRollingResistance": (), "radius_ratio": (), "elasticModulus": (),
           "poissonRatio": (), "compressiveStrength": (), "tensileStrength": (),
           "shearStrength": ()}
WALL = {"normal": (3,), "distance": (), "materialType": ()}
CONTACT = {"i": (), "j": (), "isActive": (), "isBonded": (), "materialType_i": (),
           "materialType_j": (), "position": (3,), "force_a": (3,), "moment_a": (3,),
           "moment_b": (3,), "shear_displacement": (3,)}


class Record(SimpleNamespace):
    pass


def make_record(spec: dict, **kw) -> Record:
    rec = Record()
    for name, shape in spec.items():
        setattr(rec, name, 0 if shape == () else vec(np.zeros(shape)))
    for name, v in kw.items():
        if name not in spec:
            raise KeyError(name)
        setattr(rec, name, v if spec[name] == () else vec(np.array(v, dtype=np.float64)))
    return rec


def record_type(spec: dict):
    return lambda **kw: make_record(spec, **kw)


class Field:
    """A 1-D or 2-D field of records; iterating it yields its indices."""

    def __init__(self, spec: dict, shape):
        self.spec = spec
        self.shape = tuple(shape) if isinstance(shape, (tuple, list)) else (shape,)
        self._recs = {idx: make_record(spec) for idx in itertools.product(*(range(n) for n in self.shape))}

    def _key(self, idx):
        return idx if isinstance(idx, tuple) else (idx,)

    def __getitem__(self, idx):
        return self._recs[self._key(idx)]

    def __setitem__(self, idx, rec):
        self._recs[self._key(idx)] = rec

    def __iter__(self):
        return iter(range(self.shape[0]))
