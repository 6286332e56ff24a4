"""Synthetic flowVC inputs written in ompVC's on-disk formats.

Every generator here is seeded and writes the exact binary layouts that
ompVC's loaders read:

* ``<prefix>_Cartesian.bin``: XMin XMax (f64) XRes (i32), the same for Y and Z,
  packed with no padding (ompVC/mesh.c:73-94).
* ``<prefix>_coordinates.bin``: i32 N, then N x 3 f64 (ompVC/mesh.c:135-157).
* ``<prefix>_connectivity.bin`` / ``_adjacency.bin``: i32 E, then E x 4 i32
  (ompVC/mesh.c:166-205).  Triangles use slot 3 = -1 (connectivity) and 0
  (adjacency), as the bundled Stenosis2D mesh does.
* ``<prefix>_vel.<suffix>.bin``: f64 time stamp, then (u, v, w) f64 per node,
  interleaved; Cartesian nodes in k, j, i order with i fastest
  (ompVC/velocity.c:126-141, 184-211).
* tracer seeds ``Trace_InFileFormat = 4``: i32 N, then N x Dimensions f64
  (ompVC/tracers.c:1010-1035).

Adjacency slot convention (ompVC/velocity.c:588-609, ompVC/mesh.c:552-559):
slot 0 is the face opposite node 1, slot 1 opposite node 2, slot 2 opposite
node 3 and slot 3 opposite node 0; for triangles slot 0 is the edge opposite
node 1, slot 1 opposite node 2, slot 2 opposite node 0.  -1 marks a boundary.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# ---------------------------------------------------------------- file writers


def write_cartesian_mesh(path, xmin, xmax, xres, ymin, ymax, yres, zmin, zmax, zres):
    rec = np.zeros(1, dtype=np.dtype([
        ("xmin", "<f8"), ("xmax", "<f8"), ("xres", "<i4"),
        ("ymin", "<f8"), ("ymax", "<f8"), ("yres", "<i4"),
        ("zmin", "<f8"), ("zmax", "<f8"), ("zres", "<i4")]))
    rec[0] = (xmin, xmax, xres, ymin, ymax, yres, zmin, zmax, zres)
    with open(path, "wb") as f:
        f.write(rec.tobytes())


def write_unstructured_mesh(prefix_path, xyz, conn, adj):
    xyz = np.ascontiguousarray(xyz, dtype="<f8")
    conn = np.ascontiguousarray(conn, dtype="<i4")
    adj = np.ascontiguousarray(adj, dtype="<i4")
    with open(prefix_path + "_coordinates.bin", "wb") as f:
        f.write(np.int32(xyz.shape[0]).tobytes())
        f.write(xyz.tobytes())
    with open(prefix_path + "_connectivity.bin", "wb") as f:
        f.write(np.int32(conn.shape[0]).tobytes())
        f.write(conn.tobytes())
    with open(prefix_path + "_adjacency.bin", "wb") as f:
        f.write(np.int32(adj.shape[0]).tobytes())
        f.write(adj.tobytes())


def write_frame(path, t, uvw):
    uvw = np.ascontiguousarray(uvw, dtype="<f8")
    with open(path, "wb") as f:
        f.write(np.float64(t).tobytes())
        f.write(uvw.tobytes())


def write_seed_list(path, pts, dims):
    pts = np.ascontiguousarray(np.asarray(pts, dtype="<f8")[:, :dims])
    with open(path, "wb") as f:
        f.write(np.int32(pts.shape[0]).tobytes())
        f.write(pts.tobytes())


def read_frame(path, nnodes):
    with open(path, "rb") as f:
        t = np.frombuffer(f.read(8), "<f8")[0]
        uvw = np.frombuffer(f.read(nnodes * 24), "<f8").reshape(nnodes, 3)
    return float(t), uvw


# ---------------------------------------------------------------- meshes


def kuhn_cube_mesh(n, jitter=0.2, seed=0, lo=0.0, hi=1.0):
    """Unit cube of n^3 cells, each split into 6 Kuhn tetrahedra.

    Tet (v, v+e_a, v+e_a+e_b, v+e_a+e_b+e_c) for every permutation (a, b, c)
    of the axes; the split is conforming across cells.  Interior nodes are
    displaced uniformly by +-jitter*h per coordinate with numpy's PCG64 seeded
    by ``seed``; boundary nodes stay on the lattice.  Returns (xyz, conn, adj)
    with every tetrahedron positively oriented (ompVC's determinant V > 0).
    """
    h = (hi - lo) / n
    m = n + 1
    idx = np.arange(m, dtype=np.int64)
    I, J, K = np.meshgrid(idx, idx, idx, indexing="ij")
    # node id = (i * m + j) * m + k  (k fastest)
    xyz = np.stack([lo + I * h, lo + J * h, lo + K * h], axis=-1).reshape(-1, 3)
    if jitter:
        rng = np.random.default_rng(seed)
        disp = rng.uniform(-jitter * h, jitter * h, size=xyz.shape)
        inner = ((I > 0) & (I < n) & (J > 0) & (J < n) & (K > 0) & (K < n)).reshape(-1)
        xyz[inner] += disp[inner]
    ci = np.arange(n, dtype=np.int64)
    CI, CJ, CK = np.meshgrid(ci, ci, ci, indexing="ij")
    base = np.stack([CI, CJ, CK], axis=-1).reshape(-1, 3)
    unit = np.eye(3, dtype=np.int64)
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    tets = []
    for (a, b, c) in perms:
        v0 = base
        v1 = v0 + unit[a]
        v2 = v1 + unit[b]
        v3 = v2 + unit[c]
        vs = [((v[:, 0] * m + v[:, 1]) * m + v[:, 2]) for v in (v0, v1, v2, v3)]
        tets.append(np.stack(vs, axis=-1))
    # interleave so the 6 tets of one cell are consecutive
    conn = np.stack(tets, axis=1).reshape(-1, 4)
    conn = _orient_tets(xyz, conn)
    adj = tet_adjacency(conn)
    return xyz, conn.astype(np.int32), adj


def _tet_volume(xyz, conn):
    p = xyz[conn]
    d1 = p[:, 1] - p[:, 0]
    d2 = p[:, 2] - p[:, 0]
    d3 = p[:, 3] - p[:, 0]
    return np.einsum("ij,ij->i", d1, np.cross(d2, d3))


def _orient_tets(xyz, conn):
    conn = conn.copy()
    vol = _tet_volume(xyz, conn)
    neg = vol < 0
    conn[neg, 2], conn[neg, 3] = conn[neg, 3].copy(), conn[neg, 2].copy()
    vol = _tet_volume(xyz, conn)
    if np.any(vol <= 0):
        raise ValueError(f"{int(np.sum(vol <= 0))} degenerate tetrahedra after jitter")
    return conn


# face opposite node k -> ompVC adjacency slot
_TET_FACE_SLOT = {1: 0, 2: 1, 3: 2, 0: 3}


def tet_adjacency(conn):
    """Neighbour across each face in ompVC's slot order (-1 on the boundary)."""
    conn = np.asarray(conn, dtype=np.int64)
    E = conn.shape[0]
    faces, owners, slots = [], [], []
    for opp, slot in _TET_FACE_SLOT.items():
        others = [c for c in range(4) if c != opp]
        faces.append(np.sort(conn[:, others], axis=1))
        owners.append(np.arange(E))
        slots.append(np.full(E, slot))
    faces = np.concatenate(faces)
    owners = np.concatenate(owners)
    slots = np.concatenate(slots)
    return _pair_faces(faces, owners, slots, E, 4)


def _pair_faces(faces, owners, slots, E, nslots):
    key = faces[:, 0]
    for c in range(1, faces.shape[1]):
        key = key * (faces.max() + 1) + faces[:, c]
    order = np.argsort(key, kind="stable")
    ks = key[order]
    adj = np.full((E, nslots), -1, dtype=np.int64)
    same = ks[1:] == ks[:-1]
    a = order[:-1][same]
    b = order[1:][same]
    adj[owners[a], slots[a]] = owners[b]
    adj[owners[b], slots[b]] = owners[a]
    return adj.astype(np.int32)


def tri_square_mesh(n, jitter=0.2, seed=0, lo=0.0, hi=1.0, ny=None, yhi=None):
    """Rectangle of n x ny cells split into 2 triangles each.

    Interior nodes jittered by +-jitter*h; returns (xyz, conn, adj) in ompVC's
    4-int triangle layout (connectivity slot 3 = -1, adjacency slot 3 = 0).
    """
    ny = n if ny is None else ny
    yhi = hi if yhi is None else yhi
    hx = (hi - lo) / n
    hy = (yhi - lo) / ny
    I, J = np.meshgrid(np.arange(n + 1), np.arange(ny + 1), indexing="ij")
    xyz = np.stack([lo + I * hx, lo + J * hy, np.zeros_like(I, dtype=float)], -1).reshape(-1, 3)
    if jitter:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter, jitter, size=(xyz.shape[0], 2)) * np.array([hx, hy])
        inner = ((I > 0) & (I < n) & (J > 0) & (J < ny)).reshape(-1)
        xyz[inner, :2] += d[inner]
    CI, CJ = np.meshgrid(np.arange(n), np.arange(ny), indexing="ij")
    v00 = (CI * (ny + 1) + CJ).reshape(-1)
    v10 = ((CI + 1) * (ny + 1) + CJ).reshape(-1)
    v01 = (CI * (ny + 1) + CJ + 1).reshape(-1)
    v11 = ((CI + 1) * (ny + 1) + CJ + 1).reshape(-1)
    t1 = np.stack([v00, v10, v11], -1)
    t2 = np.stack([v00, v11, v01], -1)
    tris = np.stack([t1, t2], axis=1).reshape(-1, 3)
    p = xyz[tris]
    area = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])
    if np.any(area <= 0):
        raise ValueError("degenerate triangles after jitter")
    E = tris.shape[0]
    faces, owners, slots = [], [], []
    for opp, slot in ((1, 0), (2, 1), (0, 2)):
        others = [c for c in range(3) if c != opp]
        faces.append(np.sort(tris[:, others], axis=1))
        owners.append(np.arange(E))
        slots.append(np.full(E, slot))
    adj3 = _pair_faces(np.concatenate(faces), np.concatenate(owners), np.concatenate(slots), E, 3)
    conn = np.full((E, 4), -1, dtype=np.int32)
    conn[:, :3] = tris
    adj = np.zeros((E, 4), dtype=np.int32)
    adj[:, :3] = adj3
    return xyz, conn, adj


# ---------------------------------------------------------------- flows


# ---------------------------------------------------------------- portable sine / cosine
#
# Frames are generated on more than one machine (an x86-64 host makes the
# fixtures, an aarch64 host runs the same tests), and libm's sin / cos may
# differ between them in the last bit, which a chaotic flow amplifies.  The
# analytic flows below therefore use this sine and cosine, built from
# IEEE additions and multiplications only (each a separate numpy ufunc, so
# nothing is fused): Cody-Waite reduction by pi/2 split in two parts (the
# first with 33 significant bits, so k * part exactly for the |k| < 2^20 used
# here), then the Taylor series of sin and cos on [-pi/4, pi/4] to degree
# 21 / 20 (truncation below 1e-24).  Same bytes on every IEEE machine.

_PIO2_HI = 1.57079632673412561417e+00   # pi/2 to 33 bits
_PIO2_LO = 6.07710050650619224932e-11   # pi/2 - _PIO2_HI
_SIN_C = [(-1.0) ** k / math.factorial(2 * k + 1) for k in range(11)]   # r^(2k+1)
_COS_C = [(-1.0) ** k / math.factorial(2 * k) for k in range(11)]       # r^(2k)


def _sincos(x):
    x = np.asarray(x, np.float64)
    k = np.rint(x * (2.0 / math.pi))
    r = (x - k * _PIO2_HI) - k * _PIO2_LO
    r2 = r * r
    ps = np.full_like(r, _SIN_C[-1])
    pc = np.full_like(r, _COS_C[-1])
    for cs, cc in zip(_SIN_C[-2::-1], _COS_C[-2::-1]):
        ps = ps * r2 + cs
        pc = pc * r2 + cc
    sr, cr = ps * r, pc
    q = np.mod(k, 4.0)
    sin = np.where(q == 0, sr, np.where(q == 1, cr, np.where(q == 2, -sr, -cr)))
    cos = np.where(q == 0, cr, np.where(q == 1, -sr, np.where(q == 2, -cr, sr)))
    return sin, cos


def psin(x):
    """sin(x), identical bytes on every IEEE-754 machine (|x| < 1e6)."""
    s = _sincos(x)[0]
    return float(s) if np.ndim(s) == 0 else s


def pcos(x):
    """cos(x), identical bytes on every IEEE-754 machine (|x| < 1e6)."""
    c = _sincos(x)[1]
    return float(c) if np.ndim(c) == 0 else c


def double_gyre(x, y, t, A=0.1, eps=0.25, omega=2 * math.pi / 10):
    s = eps * psin(omega * t)
    f = s * x * x + (1 - 2 * s) * x
    dfdx = 2 * s * x + (1 - 2 * s)
    u = -math.pi * A * psin(math.pi * f) * pcos(math.pi * y)
    v = math.pi * A * pcos(math.pi * f) * psin(math.pi * y) * dfdx
    return u, v


def abc_flow(xyz, t, A=math.sqrt(3), B=math.sqrt(2), C=1.0, amp=0.1):
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    g = 1.0 + amp * psin(2 * math.pi * t)
    sx, cx = _sincos(x)
    sy, cy = _sincos(y)
    sz, cz = _sincos(z)
    u = (A * sz + C * cy) * g
    v = (B * sx + A * cz) * g
    w = (C * sy + B * cx) * g
    return np.stack([u, v, w], axis=-1)


# ---------------------------------------------------------------- .in writer

# Positional key order of ompVC/parameters.c:30-138 (104 values).  Key names
# are ignored by the parser; only the order matters.
IN_KEYS = [
    ("Path_Data", "s"), ("Path_Output", "s"), ("Dimensions", "d"),
    ("Data_MeshType", "d"), ("Data_InFilePrefix", "s"), ("Data_SuffixTMin", "d"),
    ("Data_SuffixTDelta", "d"), ("Data_TRes", "d"), ("Data_TDelta", "f"),
    ("Data_TMin", "f"), ("Data_TPeriodic", "d"),
    ("Data_MeshBounds.XMin", "f"), ("Data_MeshBounds.XMax", "f"),
    ("Data_MeshBounds.YMin", "f"), ("Data_MeshBounds.YMax", "f"),
    ("Data_MeshBounds.ZMin", "f"), ("Data_MeshBounds.ZMax", "f"),
    ("Fluid_Density", "f"), ("Fluid_Viscosity", "f"),
    ("Output_TStart", "f"), ("Output_TRes", "d"), ("Output_TDelta", "f"),
    ("Int_Type", "d"), ("Int_TimeStep", "f"), ("Int_Accuracy", "f"),
    ("Int_MinTimeStep", "f"), ("Int_MaxTimeStep", "f"), ("Int_TimeDirection", "d"),
    ("Int_NormalFlow", "d"), ("Int_NormalFlowScaling", "f"), ("Int_Extrapolate", "d"),
    ("Particle_Radius", "f"), ("Particle_Density", "f"), ("Particle_ICType", "d"),
    ("Gravity_Vector[0]", "f"), ("Gravity_Vector[1]", "f"), ("Gravity_Vector[2]", "f"),
    ("LocalSearchChecking", "d"), ("Num_threads", "d"),
    ("FTLE_Compute", "d"), ("FTLE_GenerateMesh", "d"), ("FTLE_ICFile", "s"),
    ("FTLE_MeshBounds.XMin", "f"), ("FTLE_MeshBounds.XMax", "f"),
    ("FTLE_MeshBounds.YMin", "f"), ("FTLE_MeshBounds.YMax", "f"),
    ("FTLE_MeshBounds.ZMin", "f"), ("FTLE_MeshBounds.ZMax", "f"),
    ("FTLE_MeshBounds.XRes", "d"), ("FTLE_MeshBounds.YRes", "d"), ("FTLE_MeshBounds.ZRes", "d"),
    ("FTLE_IntTLength", "f"), ("FTLE_ComputeVariation", "d"), ("FTLE_VariationOutFreq", "d"),
    ("FTLE_OutFilePrefix", "s"),
    ("Trace_Compute", "d"), ("Trace_ReleaseStrategy", "d"), ("Trace_ReleaseTMax", "f"),
    ("Trace_GenerateMesh", "d"), ("Trace_InFile", "s"), ("Trace_MultipleInFiles", "d"),
    ("Trace_InFileFormat", "d"), ("Trace_OutFilePrefix", "s"), ("Trace_NumLaunchTimes", "d"),
    ("Trace_LaunchTimeSpacing", "f"), ("Trace_IntTLength", "f"), ("Trace_AlwaysOutput", "d"),
    ("Trace_MeshBounds.XMin", "f"), ("Trace_MeshBounds.XMax", "f"),
    ("Trace_MeshBounds.YMin", "f"), ("Trace_MeshBounds.YMax", "f"),
    ("Trace_MeshBounds.ZMin", "f"), ("Trace_MeshBounds.ZMax", "f"),
    ("Trace_MeshBounds.XRes", "d"), ("Trace_MeshBounds.YRes", "d"), ("Trace_MeshBounds.ZRes", "d"),
    ("Trace_APCompute", "d"), ("Trace_ComputeCET", "d"), ("Trace_CETAuxillaryMesh", "d"),
    ("Trace_CETAuxillaryMeshPrefix", "s"), ("Trace_CETSubsteps", "d"), ("Trace_ComputeRT", "d"),
    ("Trace_RTOutFilePrefix", "s"),
    ("VelOut_Compute", "d"), ("VelOut_GenerateMesh", "d"), ("VelOut_InFile", "s"),
    ("VelOut_InFileFormat", "d"), ("VelOut_FilePrefix", "s"),
    ("VelOut_MeshBounds.XMin", "f"), ("VelOut_MeshBounds.XMax", "f"),
    ("VelOut_MeshBounds.YMin", "f"), ("VelOut_MeshBounds.YMax", "f"),
    ("VelOut_MeshBounds.ZMin", "f"), ("VelOut_MeshBounds.ZMax", "f"),
    ("VelOut_MeshBounds.XRes", "d"), ("VelOut_MeshBounds.YRes", "d"), ("VelOut_MeshBounds.ZRes", "d"),
]

IN_DEFAULTS = {
    "Path_Data": "pwd", "Path_Output": "pwd", "Data_SuffixTMin": 0, "Data_SuffixTDelta": 1,
    "Data_TMin": 0.0, "Data_TPeriodic": 0, "Fluid_Density": 1.0, "Fluid_Viscosity": 1.0,
    "Output_TStart": 0.0, "Output_TRes": 1, "Output_TDelta": 1.0,
    "Int_Type": 1, "Int_TimeStep": 0.01, "Int_Accuracy": 1e-4, "Int_MinTimeStep": 1e-4,
    "Int_MaxTimeStep": 1e-3, "Int_TimeDirection": 1, "Int_NormalFlow": 0,
    "Int_NormalFlowScaling": 100.0, "Int_Extrapolate": 0, "Particle_Radius": 0.0,
    "Particle_Density": 1.0, "Particle_ICType": 0, "Gravity_Vector[0]": 0.0,
    "Gravity_Vector[1]": 0.0, "Gravity_Vector[2]": 0.0, "LocalSearchChecking": 1,
    "Num_threads": 0, "FTLE_Compute": 0, "FTLE_GenerateMesh": 1, "FTLE_ICFile": "ftle_ic.bin",
    "FTLE_MeshBounds.XMin": 0.0, "FTLE_MeshBounds.XMax": 1.0, "FTLE_MeshBounds.YMin": 0.0,
    "FTLE_MeshBounds.YMax": 1.0, "FTLE_MeshBounds.ZMin": 0.0, "FTLE_MeshBounds.ZMax": 0.0,
    "FTLE_MeshBounds.XRes": 2, "FTLE_MeshBounds.YRes": 2, "FTLE_MeshBounds.ZRes": 1,
    "FTLE_IntTLength": 1.0, "FTLE_ComputeVariation": 0, "FTLE_VariationOutFreq": 1,
    "FTLE_OutFilePrefix": "ftle", "Trace_Compute": 0, "Trace_ReleaseStrategy": 0,
    "Trace_ReleaseTMax": 0.0, "Trace_GenerateMesh": 0, "Trace_InFile": "seeds.bin",
    "Trace_MultipleInFiles": 0, "Trace_InFileFormat": 4, "Trace_OutFilePrefix": "tracer",
    "Trace_NumLaunchTimes": 1, "Trace_LaunchTimeSpacing": 0.0, "Trace_IntTLength": 1.0,
    "Trace_AlwaysOutput": 0, "Trace_MeshBounds.XMin": 0.0, "Trace_MeshBounds.XMax": 1.0,
    "Trace_MeshBounds.YMin": 0.0, "Trace_MeshBounds.YMax": 1.0, "Trace_MeshBounds.ZMin": 0.0,
    "Trace_MeshBounds.ZMax": 0.0, "Trace_MeshBounds.XRes": 1, "Trace_MeshBounds.YRes": 1,
    "Trace_MeshBounds.ZRes": 1, "Trace_APCompute": 0, "Trace_ComputeCET": 0,
    "Trace_CETAuxillaryMesh": 0, "Trace_CETAuxillaryMeshPrefix": "aux", "Trace_CETSubsteps": 2,
    "Trace_ComputeRT": 0, "Trace_RTOutFilePrefix": "rt", "VelOut_Compute": 0,
    "VelOut_GenerateMesh": 1, "VelOut_InFile": "velin.vtk", "VelOut_InFileFormat": 2,
    "VelOut_FilePrefix": "velout", "VelOut_MeshBounds.XMin": 0.0, "VelOut_MeshBounds.XMax": 1.0,
    "VelOut_MeshBounds.YMin": 0.0, "VelOut_MeshBounds.YMax": 1.0, "VelOut_MeshBounds.ZMin": 0.0,
    "VelOut_MeshBounds.ZMax": 0.0, "VelOut_MeshBounds.XRes": 1, "VelOut_MeshBounds.YRes": 1,
    "VelOut_MeshBounds.ZRes": 1,
}


def write_in_file(path, **values):
    """Write an ompVC ``.in`` file in the order ompVC's parser expects.

    Floats are written with repr() so the parser's %lf reads back the exact
    double the caller passed.
    """
    unknown = set(values) - {k for k, _ in IN_KEYS}
    if unknown:
        raise KeyError(f"unknown .in keys: {sorted(unknown)}")
    lines = ["# flowVC input file (ompVC key order)"]
    for key, typ in IN_KEYS:
        v = values.get(key, IN_DEFAULTS.get(key))
        if v is None:
            raise KeyError(f"missing value for {key}")
        if typ == "f":
            s = repr(float(v))
        elif typ == "d":
            s = str(int(v))
        else:
            s = str(v)
        lines.append(f"{key} = {s}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


# ---------------------------------------------------------------- cases


@dataclass
class Case:
    """A generated input set: directory, file prefix and its .in values."""
    root: str
    prefix: str
    params: dict = field(default_factory=dict)

    def in_path(self, name="run.in"):
        return os.path.join(self.root, name)

    def write_in(self, name="run.in", **over):
        p = dict(self.params)
        p.update(over)
        path = self.in_path(name)
        write_in_file(path, **p)
        return path


def make_double_gyre_case(root, nx=257, ny=129, nframes=101, dt=0.1, prefix="dg"):
    """Double gyre sampled on an nx x ny grid over [0,2]x[0,1], w = 0."""
    os.makedirs(root, exist_ok=True)
    write_cartesian_mesh(os.path.join(root, prefix + "_Cartesian.bin"), 0.0, 2.0, nx, 0.0, 1.0, ny, 0.0, 0.0, 1)
    xs = np.linspace(0.0, 2.0, nx)
    ys = np.linspace(0.0, 1.0, ny)
    # file order k, j, i with i fastest
    Y, X = np.meshgrid(ys, xs, indexing="ij")
    for n in range(nframes):
        t = n * dt
        u, v = double_gyre(X, Y, t)
        uvw = np.stack([u, v, np.zeros_like(u)], -1).reshape(-1, 3)
        write_frame(os.path.join(root, f"{prefix}_vel.{n}.bin"), t, uvw)
    params = dict(Path_Data=root + "/", Path_Output=root + "/", Dimensions=2, Data_MeshType=0,
                  Data_InFilePrefix=prefix, Data_SuffixTMin=0, Data_SuffixTDelta=1,
                  Data_TRes=nframes, Data_TDelta=dt, Data_TMin=0.0, Data_TPeriodic=0,
                  **{"Data_MeshBounds.XMin": 0.0, "Data_MeshBounds.XMax": 2.0,
                     "Data_MeshBounds.YMin": 0.0, "Data_MeshBounds.YMax": 1.0,
                     "Data_MeshBounds.ZMin": 0.0, "Data_MeshBounds.ZMax": 0.0})
    return Case(root, prefix, params)


def make_abc_cube_case(root, n=64, nframes=51, dt=0.02, jitter=0.2, seed=0, prefix="cube"):
    """Jittered Kuhn-cube tet mesh of [0,1]^3 with ABC velocity frames."""
    os.makedirs(root, exist_ok=True)
    xyz, conn, adj = kuhn_cube_mesh(n, jitter=jitter, seed=seed)
    write_unstructured_mesh(os.path.join(root, prefix), xyz, conn, adj)
    for f in range(nframes):
        t = f * dt
        write_frame(os.path.join(root, f"{prefix}_vel.{f}.bin"), t, abc_flow(xyz, t))
    params = dict(Path_Data=root + "/", Path_Output=root + "/", Dimensions=3, Data_MeshType=1,
                  Data_InFilePrefix=prefix, Data_SuffixTMin=0, Data_SuffixTDelta=1,
                  Data_TRes=nframes, Data_TDelta=dt, Data_TMin=0.0, Data_TPeriodic=0,
                  **{"Data_MeshBounds.XMin": 0.0, "Data_MeshBounds.XMax": 1.0,
                     "Data_MeshBounds.YMin": 0.0, "Data_MeshBounds.YMax": 1.0,
                     "Data_MeshBounds.ZMin": 0.0, "Data_MeshBounds.ZMax": 1.0})
    return Case(root, prefix, params)


def make_tri_case(root, n=32, nframes=11, dt=0.1, jitter=0.2, seed=0, prefix="tri"):
    """Jittered triangle mesh of [0,2]x[0,1] with double-gyre frames."""
    os.makedirs(root, exist_ok=True)
    xyz, conn, adj = tri_square_mesh(2 * n, jitter=jitter, seed=seed, lo=0.0, hi=2.0, ny=n, yhi=1.0)
    write_unstructured_mesh(os.path.join(root, prefix), xyz, conn, adj)
    for f in range(nframes):
        t = f * dt
        u, v = double_gyre(xyz[:, 0], xyz[:, 1], t)
        write_frame(os.path.join(root, f"{prefix}_vel.{f}.bin"), t, np.stack([u, v, np.zeros_like(u)], -1))
    params = dict(Path_Data=root + "/", Path_Output=root + "/", Dimensions=2, Data_MeshType=1,
                  Data_InFilePrefix=prefix, Data_SuffixTMin=0, Data_SuffixTDelta=1,
                  Data_TRes=nframes, Data_TDelta=dt, Data_TMin=0.0, Data_TPeriodic=0,
                  **{"Data_MeshBounds.XMin": 0.0, "Data_MeshBounds.XMax": 2.0,
                     "Data_MeshBounds.YMin": 0.0, "Data_MeshBounds.YMax": 1.0,
                     "Data_MeshBounds.ZMin": 0.0, "Data_MeshBounds.ZMax": 0.0})
    return Case(root, prefix, params)


def make_cart3d_case(root, n=17, nframes=11, dt=0.05, prefix="c3"):
    """ABC flow sampled on an n^3 Cartesian grid over [0,1]^3."""
    os.makedirs(root, exist_ok=True)
    write_cartesian_mesh(os.path.join(root, prefix + "_Cartesian.bin"), 0.0, 1.0, n, 0.0, 1.0, n, 0.0, 1.0, n)
    g = np.linspace(0.0, 1.0, n)
    Z, Y, X = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([X, Y, Z], -1).reshape(-1, 3)  # k, j, i with i fastest
    for f in range(nframes):
        t = f * dt
        write_frame(os.path.join(root, f"{prefix}_vel.{f}.bin"), t, abc_flow(pts, t))
    params = dict(Path_Data=root + "/", Path_Output=root + "/", Dimensions=3, Data_MeshType=0,
                  Data_InFilePrefix=prefix, Data_SuffixTMin=0, Data_SuffixTDelta=1,
                  Data_TRes=nframes, Data_TDelta=dt, Data_TMin=0.0, Data_TPeriodic=0,
                  **{"Data_MeshBounds.XMin": 0.0, "Data_MeshBounds.XMax": 1.0,
                     "Data_MeshBounds.YMin": 0.0, "Data_MeshBounds.YMax": 1.0,
                     "Data_MeshBounds.ZMin": 0.0, "Data_MeshBounds.ZMax": 1.0})
    return Case(root, prefix, params)


def uniform_seeds(n, dims=3, seed=0, lo=0.0, hi=1.0):
    rng = np.random.default_rng(seed)
    pts = rng.uniform(lo, hi, size=(n, 3))
    if dims == 2:
        pts[:, 2] = 0.0
    return pts


# ---------------------------------------------------------------- bent tube

def _kuhn_conn(nx, ny, nz):
    """Kuhn 6-tet split of an nx x ny x nz grid of hexahedral cells, nodes
    numbered (i * (ny+1) + j) * (nz+1) + k; conforming across cells."""
    my, mz = ny + 1, nz + 1
    CI, CJ, CK = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    base = np.stack([CI, CJ, CK], axis=-1).reshape(-1, 3).astype(np.int64)
    unit = np.eye(3, dtype=np.int64)
    tets = []
    for (a, b, c) in [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]:
        v0 = base
        v1 = v0 + unit[a]
        v2 = v1 + unit[b]
        v3 = v2 + unit[c]
        tets.append(np.stack([(v[:, 0] * my + v[:, 1]) * mz + v[:, 2] for v in (v0, v1, v2, v3)], axis=-1))
    return np.stack(tets, axis=1).reshape(-1, 4)


def _disc_map(u, v):
    """Shirley-Chiu concentric map of the square [-1, 1]^2 onto the unit disc
    (area preserving: constant Jacobian pi/4, so no cell degenerates)."""
    x, y = np.zeros_like(u), np.zeros_like(v)
    a = np.abs(u) >= np.abs(v)
    nz = (u != 0) | (v != 0)
    m = a & nz
    r = u[m]
    phi = (math.pi / 4) * v[m] / u[m]
    x[m], y[m] = r * np.cos(phi), r * np.sin(phi)
    m = ~a & nz
    r = v[m]
    phi = math.pi / 2 - (math.pi / 4) * u[m] / v[m]
    x[m], y[m] = r * np.cos(phi), r * np.sin(phi)
    return x, y


def tube_centreline(s, length=20.0, bend_radius=4.0):
    """Centre C(s), tangent T(s) and normal N(s) of a tube axis of the given
    length: straight, a 90-degree arc of bend_radius in the x-z plane, then
    straight again, with the two straight legs equally long.  The binormal
    is +y throughout."""
    s = np.asarray(s, dtype=np.float64)
    arc = 0.5 * math.pi * bend_radius
    ls = 0.5 * (length - arc)
    C = np.zeros(s.shape + (3,))
    T = np.zeros(s.shape + (3,))
    N = np.zeros(s.shape + (3,))
    m1 = s <= ls
    C[m1] = np.stack([0 * s[m1], 0 * s[m1], s[m1]], -1)
    T[m1] = (0.0, 0.0, 1.0)
    N[m1] = (1.0, 0.0, 0.0)
    m2 = (s > ls) & (s <= ls + arc)
    th = (s[m2] - ls) / bend_radius
    C[m2] = np.stack([bend_radius * (1 - np.cos(th)), 0 * th, ls + bend_radius * np.sin(th)], -1)
    T[m2] = np.stack([np.sin(th), 0 * th, np.cos(th)], -1)
    N[m2] = np.stack([np.cos(th), 0 * th, -np.sin(th)], -1)
    m3 = s > ls + arc
    d = s[m3] - (ls + arc)
    C[m3] = np.stack([bend_radius + d, 0 * d, ls + bend_radius + 0 * d], -1)
    T[m3] = (1.0, 0.0, 0.0)
    N[m3] = (0.0, 0.0, -1.0)
    return C, T, N


@dataclass
class Tube:
    """A tet-meshed bent tube: mesh arrays plus, per node, its axial position
    s, its radius r / R and the unit axial direction (for the velocity)."""
    xyz: np.ndarray
    conn: np.ndarray
    adj: np.ndarray
    s: np.ndarray
    r: np.ndarray
    tangent: np.ndarray
    radius: float
    length: float
    bend_radius: float

    def bounds(self):
        lo, hi = self.xyz.min(0), self.xyz.max(0)
        return [float(lo[0]), float(hi[0]), float(lo[1]), float(hi[1]), float(lo[2]), float(hi[2])]


def bent_tube_mesh(nc=40, nax=320, radius=1.0, bend_radius=4.0, length=20.0):
    """Tube of radius R with a 90-degree bend of radius bend_radius and axial
    length `length`: nc x nc cross-section cells (the square mapped onto the
    disc) x nax axial layers, each hexahedral cell split into 6 Kuhn
    tetrahedra (nc = 40, nax = 320: 3,072,000 tets, 539,601 nodes)."""
    t = np.linspace(-1.0, 1.0, nc + 1)
    U, V, S = np.meshgrid(t, t, np.linspace(0.0, length, nax + 1), indexing="ij")
    x, y = _disc_map(U.reshape(-1), V.reshape(-1))
    s = S.reshape(-1)
    C, T, N = tube_centreline(s, length, bend_radius)
    B = np.array([0.0, 1.0, 0.0])
    xyz = C + radius * (x[:, None] * N + y[:, None] * B)
    conn = _orient_tets(xyz, _kuhn_conn(nc, nc, nax))
    adj = tet_adjacency(conn)
    r = np.minimum(np.hypot(x, y), 1.0)
    return Tube(xyz, conn.astype(np.int32), adj, s, r, T, radius, length, bend_radius)


def womersley_profile(r, alpha=4.0):
    """Complex Womersley shape 1 - J0(i^{3/2} alpha r) / J0(i^{3/2} alpha) of
    the first harmonic at radius r / R (zero at the wall)."""
    from scipy.special import jv
    k = alpha * np.exp(0.75j * math.pi)
    return 1.0 - jv(0, k * r) / jv(0, k)


def womersley_frames(tube, nframes=101, period=1.0, peak=1.0, amp=0.5, alpha=4.0):
    """Pulsatile axial flow along the tube: a Poiseuille profile of centre-line
    speed `peak` plus a first harmonic of centre-line amplitude `amp` with
    Womersley number alpha, u(r, t) = peak (1 - r^2) + Re(a W(r) e^{2 pi i t / period}),
    directed along the local axis; no slip at the wall.  Frames at
    t = k period / (nframes - 1), k = 0 .. nframes - 1 (the last repeats the
    first, for Data_TPeriodic = 1).  Returns (times, list of N x 3 arrays)."""
    W = womersley_profile(tube.r, alpha)
    a = amp / abs(womersley_profile(np.zeros(1), alpha)[0])
    pois = peak * (1.0 - tube.r ** 2)
    times, frames = [], []
    for k in range(nframes):
        tk = k * period / (nframes - 1)
        ph = np.exp(2j * math.pi * (k % (nframes - 1)) / (nframes - 1))
        u = pois + np.real(a * W * ph)
        frames.append(u[:, None] * tube.tangent)
        times.append(tk)
    return times, frames


def tube_cross_section_seeds(tube, n, s, seed=0, margin=0.02):
    """n seeds uniformly distributed over the tube's cross-section at axial
    position s (radius up to (1 - margin) R)."""
    rng = np.random.default_rng(seed)
    rr = np.sqrt(rng.uniform(0.0, (1.0 - margin) ** 2, n))
    th = rng.uniform(0.0, 2 * math.pi, n)
    C, T, N = tube_centreline(np.full(n, float(s)), tube.length, tube.bend_radius)
    B = np.array([0.0, 1.0, 0.0])
    return C + tube.radius * ((rr * np.cos(th))[:, None] * N + (rr * np.sin(th))[:, None] * B)
