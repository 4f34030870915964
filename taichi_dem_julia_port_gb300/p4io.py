"""p4p / p4c files: the reference's particle and contact output format.

Writer: `save_single` (src/utils.jl:30-78).  Readers and comparators:
`read_p4p`, `read_p4c`, `compare_p4p`, `compare_p4c` (src/utils.jl:126-209),
with the same default tolerance rtol = sqrt(eps(Float64)) and the same
"contacts as sorted (i, j) pairs" semantics.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from pathlib import Path
from typing import IO

import numpy as np

RTOL_DEFAULT = math.sqrt(np.finfo(np.float64).eps)


def jl_float(x: float) -> str:
    """Shortest round-trip decimal in Julia's `string(::Float64)` style
    (fixed notation for 1e-4 <= |x| < 1e6, otherwise `d.ddde±x`)."""
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "Inf" if x > 0 else "-Inf"
    if x == 0.0:
        return "-0.0" if math.copysign(1.0, x) < 0 else "0.0"
    r = repr(x)
    ax = abs(x)
    if 1e-4 <= ax < 1e6:
        if "e" in r or "E" in r:
            r = np.format_float_positional(x, unique=True, trim="-")
        if "." not in r:
            r += ".0"
        return r
    mant, _, exp = np.format_float_scientific(x, unique=True, trim="-").partition("e")
    if "." not in mant:
        mant += ".0"
    return f"{mant}e{int(exp)}"


@dataclass
class P4PRecord:
    timestep: float
    id: np.ndarray       # int
    group: np.ndarray    # int
    volume: np.ndarray
    mass: np.ndarray
    pos: np.ndarray      # (n, 3)
    vel: np.ndarray      # (n, 3)


@dataclass
class P4CRecord:
    timestep: float
    i: np.ndarray        # 1-based, as written
    j: np.ndarray
    point: np.ndarray    # (c, 3)
    force: np.ndarray    # (c, 3)
    bonded: np.ndarray   # bool


def write_p4p(fh: IO[str], t: float, ids, groups, volume, mass, pos, vel) -> None:
    n = len(ids)
    fh.write("TIMESTEP PARTICLES\n")
    fh.write(f"{jl_float(t)} {n}\n")
    fh.write("ID  GROUP  VOLUME  MASS  PX  PY  PZ  VX  VY  VZ\n")
    rows = []
    for k in range(n):
        rows.append(" ".join([str(int(ids[k])), str(int(groups[k])), jl_float(volume[k]),
                              jl_float(mass[k])] + [jl_float(v) for v in pos[k]] +
                             [jl_float(v) for v in vel[k]]))
    if rows:
        fh.write("\n".join(rows) + "\n")


def write_p4c(fh: IO[str], t: float, i, j, point, force, bonded) -> None:
    """Contacts with 0-based i, j; written 1-based like the reference."""
    pairs = set()
    lines = []
    for k in range(len(i)):
        key = (int(i[k]), int(j[k]))
        if key in pairs:
            raise RuntimeError("Duplicate contact pairs!")
        pairs.add(key)
        lines.append(" ".join([str(key[0] + 1), str(key[1] + 1)] +
                              [jl_float(v) for v in point[k]] + [jl_float(v) for v in force[k]] +
                              [str(int(bool(bonded[k])))]) + "\n")
    fh.write("TIMESTEP CONTACTS\n")
    fh.write(f"{jl_float(t)} {len(lines)}\n")
    fh.write("P1  P2  CX  CY  CZ  FX  FY  FZ  CONTACT_IS_BONDED\n")
    fh.write("".join(lines))


def read_p4p(path: str | Path) -> list[P4PRecord]:
    lines = Path(path).read_text().splitlines()
    recs = []
    k = 0
    while k < len(lines):
        if not lines[k].strip():
            k += 1
            continue
        assert lines[k].startswith("TIMESTEP"), f"line {k + 1}: expected TIMESTEP"
        ts, n = lines[k + 1].split()[:2]
        n = int(float(n))
        data = np.array([[float(x) for x in lines[k + 3 + r].split()[:10]] for r in range(n)],
                        dtype=np.float64).reshape(n, 10)
        recs.append(P4PRecord(float(ts), data[:, 0].astype(np.int64), data[:, 1].astype(np.int64),
                              data[:, 2].copy(), data[:, 3].copy(), data[:, 4:7].copy(),
                              data[:, 7:10].copy()))
        k += 3 + n
    return recs


def read_p4c(path: str | Path) -> list[P4CRecord]:
    lines = Path(path).read_text().splitlines()
    recs = []
    k = 0
    while k < len(lines):
        if not lines[k].strip():
            k += 1
            continue
        assert lines[k].startswith("TIMESTEP"), f"line {k + 1}: expected TIMESTEP"
        ts, n = lines[k + 1].split()[:2]
        n = int(float(n))
        rows = {}
        for r in range(n):
            v = [float(x) for x in lines[k + 3 + r].split()[:9]]
            rows[(int(v[0]), int(v[1]))] = v
        keys = sorted(rows)
        arr = np.array([rows[q] for q in keys], dtype=np.float64).reshape(len(keys), 9)
        recs.append(P4CRecord(float(ts), arr[:, 0].astype(np.int64), arr[:, 1].astype(np.int64),
                              arr[:, 2:5].copy(), arr[:, 5:8].copy(), arr[:, 8] != 0))
        k += 3 + n
    return recs


def _by_id(rec: P4PRecord) -> np.ndarray:
    return np.argsort(rec.id, kind="stable")


def compare_p4p(a, b, atol: float = 0.0, rtol: float | None = None) -> None:
    """Raises AssertionError on the first mismatch (src/utils.jl:170-189)."""
    ra = read_p4p(a) if isinstance(a, (str, Path)) else a
    rb = read_p4p(b) if isinstance(b, (str, Path)) else b
    rtol = (0.0 if atol > 0 else RTOL_DEFAULT) if rtol is None else rtol
    assert len(ra) == len(rb), f"{len(ra)} vs {len(rb)} records"
    for t, (x, y) in enumerate(zip(ra, rb)):
        assert x.timestep == y.timestep, f"[timestep] record {t}"
        assert len(x.id) == len(y.id), f"[length] record {t}"
        ox, oy = _by_id(x), _by_id(y)
        assert np.array_equal(x.id[ox], y.id[oy]), f"[pid] record {t}"
        for name in ("volume", "mass", "pos", "vel"):
            u, v = getattr(x, name)[ox], getattr(y, name)[oy]
            _isapprox(u, v, atol, rtol, f"[{name}] record {t}")


def compare_p4c(a, b, atol: float = 0.0, rtol: float | None = None) -> None:
    """Raises AssertionError on the first mismatch (src/utils.jl:191-209)."""
    ra = read_p4c(a) if isinstance(a, (str, Path)) else a
    rb = read_p4c(b) if isinstance(b, (str, Path)) else b
    rtol = (0.0 if atol > 0 else RTOL_DEFAULT) if rtol is None else rtol
    assert len(ra) == len(rb), f"{len(ra)} vs {len(rb)} records"
    for t, (x, y) in enumerate(zip(ra, rb)):
        assert x.timestep == y.timestep, f"[timestep] record {t}"
        assert len(x.i) == len(y.i), f"[length] record {t}: {len(x.i)} vs {len(y.i)}"
        assert np.array_equal(x.i, y.i) and np.array_equal(x.j, y.j), f"[pair] record {t}"
        _isapprox(x.point, y.point, atol, rtol, f"[position] record {t}")
        _isapprox(x.force, y.force, atol, rtol, f"[force] record {t}")
        assert np.array_equal(x.bonded, y.bonded), f"[bonded] record {t}"


def _isapprox(u: np.ndarray, v: np.ndarray, atol: float, rtol: float, what: str) -> None:
    """Julia `isapprox` per row: norm(u - v) <= max(atol, rtol * max(norm(u), norm(v)))."""
    u = np.asarray(u, dtype=np.float64)
    v = np.asarray(v, dtype=np.float64)
    if u.ndim == 1:
        u, v = u[:, None], v[:, None]
    d = np.linalg.norm(u - v, axis=1)
    lim = np.maximum(atol, rtol * np.maximum(np.linalg.norm(u, axis=1), np.linalg.norm(v, axis=1)))
    bad = np.nonzero(~(d <= lim))[0]
    assert bad.size == 0, f"{what}: row {bad[0] if bad.size else -1}, {u[bad[:1]]} vs {v[bad[:1]]}"
