"""Wavefront OBJ / MTL parsing with the rules of the reference's objloader::simple
(src/objloader/objloader_simple.cpp:24-264).

* ``v``, ``vn``, ``vt``: positions, normals, texture coordinates (``vt`` keeps its first two values).
* ``f``: up to four vertices ``p``, ``p/t``, ``p//n`` or ``p/t/n``; a fourth vertex adds the
  triangle (0, 2, 3); further vertices are ignored. Indices are 1-based, negative ones count back
  from the current end, 0 means "absent" (-1).
* ``g`` and ``usemtl`` start a new primitive unless the current one has no faces yet; a
  primitive keeps the material that was current when it started (``usemtl`` sets it).
* ``mtllib``: a .mtl file next to the .obj; ``newmtl`` entries with ``Kd``, ``Ks``, ``Ni``, ``Ns``,
  ``aniso``, ``Ke``, ``illum``, ``map_Kd``; fields not given are 0 (empty for ``map_Kd``).
* Without any material a single ``default`` material (illum -1, Kd 1) is used.

A command matches when its name is followed by a space or tab, as in the reference.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np


@dataclass
class MTLMaterial:
    name: str
    illum: int = 0
    Kd: tuple = (0.0, 0.0, 0.0)
    Ks: tuple = (0.0, 0.0, 0.0)
    Ke: tuple = (0.0, 0.0, 0.0)
    map_Kd: str = ""
    Ni: float = 0.0
    Ns: float = 0.0
    an: float = 0.0


@dataclass
class OBJPrimitive:
    material: int = 0
    faces: list = field(default_factory=list)  # (p, t, n) index triples, three per triangle


@dataclass
class OBJModel:
    ps: np.ndarray
    ns: np.ndarray
    ts: np.ndarray
    primitives: list
    materials: list


def _command(line: str, name: str) -> bool:
    n = len(name)
    return line.startswith(name) and len(line) > n and line[n] in " \t"


def _floats(s: str, k: int) -> list:
    """The first k numbers of s, as atof would read them (missing ones are 0)."""
    out = []
    for tok in s.split()[:k]:
        try:
            out.append(float(tok.split("/")[0]))
        except ValueError:
            out.append(0.0)
    return out + [0.0] * (k - len(out))


def _atoi(s: str) -> int:
    s = s.strip()
    j = 1 if s[:1] in "+-" else 0
    while j < len(s) and s[j].isdigit():
        j += 1
    try:
        return int(s[:j])
    except ValueError:
        return 0


def _index(i: int, n: int) -> int:
    return n + i if i < 0 else (i - 1 if i > 0 else -1)


def _vertex(tok: str, counts) -> tuple:
    parts = tok.split("/")
    p = _index(_atoi(parts[0]), counts[0])
    t = _index(_atoi(parts[1]), counts[2]) if len(parts) > 1 else -1
    n = _index(_atoi(parts[2]), counts[1]) if len(parts) > 2 else -1
    return p, t, n


def load_mtl(path: str, materials: list, index: dict) -> None:
    with open(path, "r", errors="replace") as f:
        for raw in f:
            line = raw.lstrip(" \t").rstrip("\r\n")
            if _command(line, "newmtl"):
                name = line[7:].split()[0] if line[7:].split() else ""
                index[name] = len(materials)
                materials.append(MTLMaterial(name))
                continue
            if not materials:
                continue
            m = materials[-1]
            if _command(line, "Kd"):
                m.Kd = tuple(_floats(line[3:], 3))
            elif _command(line, "Ks"):
                m.Ks = tuple(_floats(line[3:], 3))
            elif _command(line, "Ni"):
                m.Ni = _floats(line[3:], 1)[0]
            elif _command(line, "Ns"):
                m.Ns = _floats(line[3:], 1)[0]
            elif _command(line, "aniso"):
                m.an = _floats(line[6:], 1)[0]
            elif _command(line, "Ke"):
                m.Ke = tuple(_floats(line[3:], 3))
            elif _command(line, "illum"):
                m.illum = _atoi(line[6:])
            elif _command(line, "map_Kd"):
                toks = line[7:].split()
                m.map_Kd = toks[0] if toks else ""


def load_obj(path: str) -> OBJModel:
    """Parses an .obj file (and the .mtl files it names). Raises OSError if a file is missing and
    ValueError on an unknown material name, where the reference's loader fails."""
    ps, ns, ts = [], [], []
    prims: list[OBJPrimitive] = []
    materials: list[MTLMaterial] = []
    index: dict[str, int] = {}
    cur = 0
    base = os.path.dirname(os.path.abspath(path))
    with open(path, "r", errors="replace") as f:
        for raw in f:
            line = raw.lstrip(" \t").rstrip("\r\n")
            if _command(line, "v"):
                ps.append(_floats(line[2:], 3))
            elif _command(line, "vn"):
                ns.append(_floats(line[3:], 3))
            elif _command(line, "vt"):
                ts.append(_floats(line[3:], 3)[:2])
            elif _command(line, "g"):
                if not prims or prims[-1].faces:
                    prims.append(OBJPrimitive())
                prims[-1].material = cur
            elif _command(line, "f"):
                if not prims:
                    prims.append(OBJPrimitive())
                counts = (len(ps), len(ns), len(ts))
                vs = [_vertex(tok, counts) for tok in line[2:].split()[:4]]
                if len(vs) < 3:
                    continue
                prims[-1].faces.extend([vs[0], vs[1], vs[2]])
                if len(vs) == 4 and vs[3][0] != -1:
                    prims[-1].faces.extend([vs[0], vs[2], vs[3]])
            elif _command(line, "usemtl"):
                toks = line[7:].split()
                name = toks[0] if toks else ""
                if not prims or prims[-1].faces:
                    prims.append(OBJPrimitive())
                if name not in index:
                    raise ValueError(f"Invalid material [name='{name}']")
                cur = index[name]
                prims[-1].material = cur
            elif _command(line, "mtllib"):
                toks = line[7:].split()
                load_mtl(os.path.join(base, toks[0] if toks else ""), materials, index)
    if not materials:
        materials.append(MTLMaterial("default", illum=-1, Kd=(1.0, 1.0, 1.0)))
    return OBJModel(np.asarray(ps, np.float64).reshape(-1, 3), np.asarray(ns, np.float64).reshape(-1, 3),
                    np.asarray(ts, np.float64).reshape(-1, 2), prims, materials)


def init(name: str = "simple", prop: dict | None = None) -> None:
    """lm.objloader.init: the reference selects objloader::simple or objloader::tinyobjloader; the
    GPU path's model::wavefrontobj always parses with this module (the objloader::simple rules)."""


def shutdown() -> None:
    """lm.objloader.shutdown: nothing to release."""
