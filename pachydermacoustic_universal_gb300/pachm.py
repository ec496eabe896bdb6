"""The .pachm map results file of Pachyderm (Utilities.FileIO.Write_pachm / Read_pachm,
Pachyderm_Acoustic_Universal/Classes_IO.cs:263-630), so the reference's host opens the maps the GPU
engine computed, and maps it wrote load here.

Layout (.NET BinaryWriter, as in .pac1): data type string ("Type;Map_Data_NoDir"), sample count,
sample rate and receiver count (uint32); "Version" + version string; "Mesh Information",
"Mesh Vertices", vertex and face counts (uint32), vertices (3 doubles), "Mesh Faces" + 4 uint32
per face (a triangle repeats its third index); "SourceswLoc" + source count (int32) and per source
origin (3 doubles), type string and delay (double); "Receiver Hit Data" + on-vertex flag (bool),
then per source and receiver its index (uint32), direct arrival time and rho c (doubles), per band
the band index (uint32) and per sample energy and pressure (doubles), "End_Receiver_Hits";
"End_of_File".  The reader takes the receivers from the mesh (face centroids or vertices, without
the placement offset) as the reference's reader does, and the v2.5+ layout (pressure stored).
Directional maps ("Type;Map_Data") add six doubles per sample after the pressure, the +x +y +z and
-x -y -z arrival sums, as the reference's writer writes them; the reference's reader takes those six
as singles (ReadSingle) and so misreads its own directional files -- this reader takes doubles.
"""
from __future__ import annotations

import numpy as np

from .mapping import Map_Receiver, MapMesh, PachMapReceiver
from .pac1 import VERSION, _Reader, _Writer


def write_pachm(filename, maps):
    """Write_pachm (Classes_IO.cs:263-419): maps = one PachMapReceiver per source, all on one mesh."""
    m0 = maps[0]
    mesh = m0.Map_Mesh
    M = m0.Count
    with open(filename, "wb") as f:
        w = _Writer(f)
        w.string(m0.Data_Type())
        w.uint32(m0.SampleCT)
        w.uint32(m0.SampleRate)
        w.uint32(M)
        w.string("Version")
        w.string(VERSION)
        w.string("Mesh Information")
        w.string("Mesh Vertices")
        w.uint32(mesh.Vertex_Count)
        w.uint32(mesh.Polygon_Count)
        w.doubles(mesh.vertices.reshape(-1))
        w.string("Mesh Faces")
        for face in mesh.faces:
            for k in (0, 1, 2):
                w.uint32(face[k])
            w.uint32(face[3] if len(face) > 3 else face[2])
        w.string("SourceswLoc")
        w.int32(len(maps))
        for m in maps:
            for x in m.Src:
                w.double(x)
            w.string(m.SrcType)
            w.double(m.delay_ms)
        w.string("Receiver Hit Data")
        w.boolean(m0.Rec_Vertex)
        n = m0.SampleCT
        for m in maps:
            for i in range(M):
                w.uint32(i)
                w.double(m.Rec_List[i].Direct_Time)
                w.double(m0.Rec_List[i].Rho_C)
                for o in range(8):
                    w.uint32(o)
                    rec = np.empty((n, 8 if m0.Directional else 2))
                    rec[:, 0] = m._E[i, o, :n]
                    rec[:, 1] = m._P[i, o, :n]
                    if m0.Directional:
                        rec[:, 2:5] = m._Dp[i, :, o, :n].T
                        rec[:, 5:8] = m._Dn[i, :, o, :n].T
                    w.doubles(rec.reshape(-1))
                w.string("End_Receiver_Hits")
        w.string("End_of_File")


def read_pachm(filename):
    """Read_pachm (Classes_IO.cs:421-630): a list of PachMapReceiver, one per source."""
    with open(filename, "rb") as f:
        r = _Reader(f.read())
    calc = r.string()
    if calc not in ("Type;Map_Data", "Type;Map_Data_NoDir"):
        raise ValueError("Map Data File Expected")
    directional = calc == "Type;Map_Data"
    SampleCT = r.uint32()
    SampleRate = r.uint32()
    Rec_CT = r.uint32()
    version, rev = 1.1, 0
    mesh = None
    maps = None
    while True:
        tag = r.string()
        if tag == "Version":
            v = r.string()
            version = float(v[:3])
            rev = int(v.split(".")[3])
        elif tag == "Mesh Information":
            if r.string() != "Mesh Vertices":
                raise ValueError("Mesh Vertices Expected")
            VC, FC = r.uint32(), r.uint32()
            verts = r.doubles(3 * VC).reshape(VC, 3)
            if r.string() != "Mesh Faces":
                raise ValueError("Mesh Faces Expected")
            faces = []
            for _ in range(FC):
                F = [r.uint32() for _ in range(4)]
                faces.append(tuple(F[:3]) if F[2] == F[3] else tuple(F))
            mesh = MapMesh(verts, faces)
        elif tag in ("Sources", "SourceswLoc"):
            s_ct = r.int32()
            maps = []
            for _ in range(s_ct):
                m = PachMapReceiver()
                m.SampleCT, m.SampleRate, m.Map_Mesh = SampleCT, SampleRate, mesh
                m.CutOffTime = SampleCT / SampleRate * (1000.0 if tag == "SourceswLoc" else 1.0)
                m.Src = tuple(r.doubles(3)) if tag == "SourceswLoc" else (0.0, 0.0, 0.0)
                m.SrcType = r.string()
                if version > 2.0 or (version == 2.0 and rev >= 1):
                    m.delay_ms = r.double()
                maps.append(m)
        elif tag == "Receiver Hit Data":
            if maps is None:
                m = PachMapReceiver()
                m.SampleCT, m.SampleRate, m.Map_Mesh = SampleCT, SampleRate, mesh
                m.CutOffTime = SampleCT / SampleRate
                m.SrcType = "Geodesic"
                m.Src = (0.0, 0.0, 0.0)
                maps = [m]
            on_vertex = r.boolean()
            for m in maps:
                m.Rec_Vertex = on_vertex
                m.increment = 0.0
                m.Time1Pt = SampleCT == 1
                m.Directional = directional
                m._alloc(Rec_CT, SampleCT)
                m.Rec_List = []
                for i in range(Rec_CT):
                    r.uint32()
                    if version >= 1.7:
                        direct = r.double()
                    else:
                        direct = np.linalg.norm(np.subtract(m.Src, _location(mesh, on_vertex, i))) / 343.0
                    rho_c = r.double() if version >= 2.0 else 400.0
                    m.Rec_List.append(Map_Receiver(m, i, _location(mesh, on_vertex, i), direct, rho_c))
                    for o in range(8):
                        if r.uint32() != o:
                            raise ValueError(f"Octave {o} Expected")
                        npr = 2 if version >= 2.5 else 1
                        per = npr + (6 if directional else 0)
                        vals = r.doubles(per * SampleCT).reshape(SampleCT, per)
                        m._E[i, o] = vals[:, 0]
                        if version >= 2.5:
                            m._P[i, o] = vals[:, 1]
                        if directional:
                            m._Dp[i, :, o] = vals[:, npr:npr + 3].T
                            m._Dn[i, :, o] = vals[:, npr + 3:npr + 6].T
                    if r.string() != "End_Receiver_Hits":
                        raise ValueError("End of Receiver Hits Expected")
        elif tag == "End_of_File":
            return maps
        else:
            raise ValueError(f"unexpected section {tag!r}")


def _location(mesh, on_vertex, i):
    if on_vertex:
        return mesh.vertices[i]
    return mesh.Polygon_Vertices(i).mean(axis=0)
