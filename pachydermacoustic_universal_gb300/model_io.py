"""Pachyderm's text model file (Utilities.FileIO.ReadModelFile,
Pachyderm_Acoustic_Universal/Classes_IO.cs:632-902) to a scene for the GPU engine, and the writer of
the same format.

Format: '#' comments; [VERTICES] lines "id x y z"; [MATERIALS] lines "id name" each followed by
ABSORPTION=8 values, SCATTERING=..., TRANSMISSION=... (comma separated, missing ones zero, short
lists zero-padded to 8) and [END]; [OBJECT m] starts an object of material m (1-based) whose lines
"POLY v1,v2,...[ CURVE=k1,k2 FRAME=ax,ay,az,bx,by,bz]" list its polygons by vertex id.

As the reference reader does, the scene is made with 20 degC, 50 % RH, a pressure argument of 101325
passed where the Scene ctor expects hPa (so the air absorption is that of 100x atmospheric
pressure), Air_Choice 0 and edge correction on.  Curvature and frame data are parsed and checked
(curvature needs both axes and the axes need curvature) but the engine traces polygons as flat.
"""
from __future__ import annotations

import numpy as np

from .simulation import Basic_Material, Lambert_Scattering, Polygon_Scene


def _values(text):
    v = [float(s.strip()) for s in text.split(",")]
    return (v + [0.0] * 8)[:8]


def parse_model(text: str):
    """(vertices {id: xyz}, materials {id: (name, abs, scat, trans)}, objects [(material id, [[vertex ids]],
    [curvature], [frames])])."""
    vertices, materials, objects = {}, {}, []
    section = None
    lines = iter(text.splitlines())
    for raw in lines:
        line = raw.strip()
        if not line or line.startswith("#"):
            continue
        up = line.upper()
        if up.startswith("[VERTICES]"):
            section = "VERTICES"
            continue
        if up.startswith("[MATERIALS]"):
            section = "MATERIALS"
            continue
        if up.startswith("[OBJECT"):
            section = "OBJECT"
            parts = line[7:].strip().rstrip("]").split()
            if parts:
                objects.append((int(parts[0]) - 1, [], [], []))
            continue
        if section == "VERTICES":
            p = line.split()
            if len(p) >= 4:
                vertices[int(p[0])] = (float(p[1]), float(p[2]), float(p[3]))
        elif section == "MATERIALS":
            p = line.split()
            if len(p) >= 2:
                mid, name = int(p[0]), p[1]
                ab, sc, tr = [0.0] * 8, [0.0] * 8, [0.0] * 8
                for praw in lines:
                    pl = praw.strip()
                    if not pl or pl.startswith("#"):
                        continue
                    if pl.upper().startswith("[END]"):
                        break
                    if "=" in pl:
                        key, val = pl.split("=", 1)
                        key = key.strip().upper()
                        if key == "ABSORPTION":
                            ab = _values(val)
                        elif key == "SCATTERING":
                            sc = _values(val)
                        elif key == "TRANSMISSION":
                            tr = _values(val)
                materials[mid - 1] = (name, ab, sc, tr)
        elif section == "OBJECT" and objects and up.startswith("POLY"):
            parts = line[4:].split()
            if not parts:
                continue
            ids = [int(s) for s in parts[0].split(",")]
            kurv, frame = [0.0, 0.0], None
            for prop in parts[1:]:
                if prop.upper().startswith("CURVE="):
                    vals = prop[6:].split(",")
                    if len(vals) == 2:
                        kurv = [float(vals[0]), float(vals[1])]
                elif prop.upper().startswith("FRAME="):
                    vals = prop[6:].split(",")
                    if len(vals) == 6:
                        frame = [float(x) for x in vals]
            axes_zero = frame is None or (not any(frame[:3]) or not any(frame[3:]))
            if (kurv[0] or kurv[1]) and axes_zero:
                raise ValueError("Polygon has curvature but missing frame axes")
            if frame is not None and (any(frame[:3]) or any(frame[3:])) and not (kurv[0] or kurv[1]):
                raise ValueError("Polygon has frame axes but missing curvature")
            objects[-1][1].append(ids)
            objects[-1][2].append(kurv)
            objects[-1][3].append(frame)
    return vertices, materials, objects


def read_model_file(path) -> Polygon_Scene:
    """ReadModelFile: a constructed Polygon_Scene (partition it, or let the tracer do so)."""
    with open(path) as f:
        vertices, materials, objects = parse_model(f.read())
    model, mats, scats, trans = [], [], [], []
    for mid, polys, _, _ in objects:
        name, ab, sc, tr = materials.get(mid, ("", [0.0] * 8, [0.0] * 8, [0.0] * 8))
        mats.append(Basic_Material(ab))
        scats.append(Lambert_Scattering(sc))
        trans.append(np.asarray(tr))
        model.append([np.asarray([vertices[i] for i in ids]) for ids in polys])
    scene = Polygon_Scene(20.0, 50.0, 101325.0, 0, True, False)
    scene.Construct(model, mats, scats, trans)
    return scene


def write_model_file(path, arrays, materials=None):
    """Write scene arrays (rooms.SceneArrays) in the text format: one material and one object per
    distinct (absorption, scattering, transmission) row."""
    rows = np.concatenate([arrays.absorption, arrays.scattering, arrays.transmission], axis=1)
    uniq, inv = np.unique(rows, axis=0, return_inverse=True)
    inv = np.asarray(inv).reshape(-1)
    out = ["# Pachyderm model", "[VERTICES]"]
    out += [f"{i + 1} {x!r} {y!r} {z!r}" for i, (x, y, z) in enumerate(arrays.vertices.tolist())]
    out.append("[MATERIALS]")
    for m, r in enumerate(uniq):
        name = materials[m] if materials else f"material_{m + 1}"
        out.append(f"{m + 1} {name}")
        out.append("ABSORPTION=" + ",".join(repr(float(x)) for x in r[0:8]))
        out.append("SCATTERING=" + ",".join(repr(float(x)) for x in r[8:16]))
        out.append("TRANSMISSION=" + ",".join(repr(float(x)) for x in r[16:24]))
        out.append("[END]")
    for m in range(len(uniq)):
        out.append(f"[OBJECT {m + 1}]")
        for p in np.nonzero(inv == m)[0]:
            ids = arrays.poly_indices[arrays.poly_offsets[p]:arrays.poly_offsets[p + 1]] + 1
            out.append("POLY " + ",".join(str(int(i)) for i in ids))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
