"""Reader of the CGNS meshes of Phase's cases (ADF containers), with the
semantics of CgnsUnstructuredGrid::load
(src/2D/Unstructured/FiniteVolumeGrid2D/CgnsUnstructuredGrid.cpp:13-96):

* base 1 must have cell dimension 2 and one zone, of type Unstructured;
* every element of every section is gathered by its element id
  (CgnsFile::readSection, src/System/CgnsFile.cpp:183-240: BAR_2, TRI_3,
  QUAD_4 and MIXED sections);
* node coordinates are CoordinateX / CoordinateY plus the grid origin;
* a boundary condition's patch is the node list of the elements its
  PointRange or PointList names, taken two nodes at a time as faces
  (FiniteVolumeGrid2D::createPatchByNodes, FiniteVolumeGrid2D.cpp:183-198);
* the cells are the elements with more than two nodes, in element-id order.

The container is read directly (no CGNS or HDF5 library is involved): an
ADF file is a sequence of 4096-byte blocks; a file address is written as 8
hex digits of block number and 4 of byte offset; a node header ("NoDe" ..
"TaiL", 246 bytes) holds the node's name and label (32 characters each),
its child count, the address of its sub-node table ("SNTb": 32-character
name + address per child), its data type (I4, I8, R4, R8, C1 or MT), up to
12 dimensions (8 hex digits each, first index fastest) and the address of
its data chunk ("DaTa", the address of its end, the raw values).  The byte
order is the one the file header names (L little-, B big-endian).
"""
from __future__ import annotations

import numpy as np

BLOCK = 4096
# ElementType_t values of the CGNS standard (SIDS) that Phase reads
BAR_2, TRI_3, QUAD_4, MIXED = 3, 5, 7, 20
NODES_OF = {BAR_2: 2, TRI_3: 3, QUAD_4: 4}


class CgnsError(ValueError):
    """A file Phase's loader would reject, or that this reader cannot read."""


class AdfNode:
    __slots__ = ("addr", "name", "label", "n_children", "table", "dtype",
                 "dims", "n_chunks", "data_addr")


class AdfFile:
    """The node tree of an ADF container."""

    def __init__(self, path_or_bytes):
        if isinstance(path_or_bytes, (bytes, bytearray)):
            self.buf = bytes(path_or_bytes)
        else:
            with open(path_or_bytes, "rb") as f:
                self.buf = f.read()
        head = self.buf[:256]
        if b"ADF Database Version" not in head:
            raise CgnsError("not an ADF file (an HDF5-based CGNS file needs "
                            "the HDF5 library)")
        k = head.find(b"AdF2")
        order = head[k + 4:k + 5] if k >= 0 else b"L"
        self.endian = ">" if order == b"B" else "<"
        k = head.find(b"AdF4")
        if k < 0:
            raise CgnsError("ADF header without a root-node address")
        self.root = self.node(self.addr(head[k + 4:k + 16]))

    @staticmethod
    def addr(field: bytes) -> int:
        return int(field[:8], 16) * BLOCK + int(field[8:12], 16)

    def node(self, addr: int) -> AdfNode:
        h = self.buf[addr:addr + 246]
        if len(h) < 246 or h[:4] != b"NoDe" or h[242:246] != b"TaiL":
            raise CgnsError(f"no node header at byte {addr}")
        n = AdfNode()
        n.addr = addr
        n.name = h[4:36].decode("ascii").rstrip(" \x00")
        n.label = h[36:68].decode("ascii").rstrip(" \x00")
        n.n_children = int(h[68:76], 16)
        n.table = self.addr(h[84:96])
        n.dtype = h[96:128].decode("ascii").strip()
        nd = int(h[128:130], 16)
        n.dims = [int(h[130 + 8 * i:138 + 8 * i], 16) for i in range(nd)]
        n.n_chunks = int(h[226:230], 16)
        n.data_addr = self.addr(h[230:242])
        return n

    def children(self, n: AdfNode):
        if n.n_children == 0:
            return []
        t = n.table
        if self.buf[t:t + 4] != b"SNTb":
            raise CgnsError(f"no sub-node table for {n.name!r}")
        out = []
        p = t + 16  # tag + the table's end address
        for _ in range(n.n_children):
            out.append(self.node(self.addr(self.buf[p + 32:p + 44])))
            p += 44
        return out

    def child(self, n: AdfNode, name=None, label=None):
        for c in self.children(n):
            if (name is None or c.name == name) and (label is None or c.label == label):
                return c
        return None

    def data(self, n: AdfNode):
        if n.dtype == "MT" or n.n_chunks == 0:
            return None
        if n.n_chunks != 1:
            raise CgnsError(f"{n.name!r}: data in {n.n_chunks} chunks is not "
                            "read by this reader")
        a = n.data_addr
        if self.buf[a:a + 4] != b"DaTa":
            raise CgnsError(f"{n.name!r}: no data chunk at byte {a}")
        count = int(np.prod(n.dims)) if n.dims else 1
        if n.dtype == "C1":
            return self.buf[a + 16:a + 16 + count].decode("ascii").rstrip(" \x00")
        kinds = {"I4": "i4", "I8": "i8", "R4": "f4", "R8": "f8", "U4": "u4",
                 "U8": "u8"}
        if n.dtype not in kinds:
            raise CgnsError(f"{n.name!r}: data type {n.dtype} is not read")
        dt = np.dtype(self.endian + kinds[n.dtype])
        v = np.frombuffer(self.buf, dt, count, a + 16)
        # dimensions are stored first index fastest (Fortran order)
        return v.reshape(n.dims[::-1]).T if len(n.dims) > 1 else v.copy()


def _section(f: AdfFile, sec: AdfNode):
    """(start, end, node lists) of an Elements_t node
    (CgnsFile::readSection)."""
    etype, _nbndry = (int(x) for x in f.data(sec)[:2])
    rng = f.child(sec, name="ElementRange")
    con = f.child(sec, name="ElementConnectivity")
    if rng is None or con is None:
        raise CgnsError(f"section {sec.name!r} without ElementRange / "
                        "ElementConnectivity")
    start, end = (int(x) for x in np.asarray(f.data(rng)).ravel()[:2])
    conn = np.asarray(f.data(con)).ravel().astype(np.int64)
    elems = []
    if etype == MIXED:
        i = 0
        while i < conn.size:
            t = int(conn[i])
            if t not in NODES_OF:
                raise CgnsError(f"unsupported element type {t} in a MIXED "
                                "section")
            nv = NODES_OF[t]
            elems.append(conn[i + 1:i + 1 + nv])
            i += 1 + nv
    else:
        if etype not in NODES_OF:
            raise CgnsError(f"unsupported element type {etype} in section "
                            f"{sec.name!r}")
        nv = NODES_OF[etype]
        for e in range(end - start + 1):
            elems.append(conn[nv * e:nv * (e + 1)])
    if len(elems) != end - start + 1:
        raise CgnsError(f"section {sec.name!r}: {len(elems)} elements for "
                        f"the range {start}..{end}")
    return start, end, elems


def read_mesh(path_or_bytes, origin=(0.0, 0.0)):
    """The grid of a CGNS file as Phase's CgnsUnstructuredGrid loads it:
    dict(nodes [n, 2], cptr, cind (cells, 0-based node ids, element-id
    order), patches {name: [node, node, node, node, ...]} (faces as node
    pairs), base, zone names)."""
    f = AdfFile(path_or_bytes)
    bases = [c for c in f.children(f.root) if c.label == "CGNSBase_t"]
    if not bases:
        raise CgnsError("no CGNSBase_t node")
    base = bases[0]
    cell_dim, _phys_dim = (int(x) for x in f.data(base)[:2])
    if cell_dim != 2:
        raise CgnsError("cell dimension must be 2")
    zones = [c for c in f.children(base) if c.label == "Zone_t"]
    if len(zones) != 1:
        raise CgnsError("multiple zones are not supported" if zones
                        else "no zone")
    zone = zones[0]
    zt = f.child(zone, label="ZoneType_t")
    if zt is None or f.data(zt) != "Unstructured":
        raise CgnsError('zone type must be "Unstructured"')
    # elements of every section by element id
    adj = {}
    for sec in f.children(zone):
        if sec.label != "Elements_t":
            continue
        start, end, elems = _section(f, sec)
        for k, e in enumerate(elems):
            adj[start + k] = e
    if not adj:
        raise CgnsError("no element sections")
    n_elem = max(adj)
    eptr = [0]
    eind = []
    for eid in range(1, n_elem + 1):
        e = adj.get(eid, ())
        eind.extend(int(v) - 1 for v in e)
        eptr.append(len(eind))
    eptr = np.asarray(eptr, np.int64)
    eind = np.asarray(eind, np.int64)
    gc = f.child(zone, label="GridCoordinates_t")
    if gc is None:
        raise CgnsError("no GridCoordinates")
    x = np.asarray(f.data(f.child(gc, name="CoordinateX")), np.float64)
    y = np.asarray(f.data(f.child(gc, name="CoordinateY")), np.float64)
    nodes = np.stack([x + origin[0], y + origin[1]], axis=1)
    patches = {}
    zbc = f.child(zone, label="ZoneBC_t")
    for bc in (f.children(zbc) if zbc is not None else []):
        if bc.label != "BC_t":
            continue
        pr = f.child(bc, name="PointRange")
        pl = f.child(bc, name="PointList")
        if pr is not None:
            lo, hi = (int(v) for v in np.asarray(f.data(pr)).ravel()[:2])
            elems = range(lo, hi + 1)
        elif pl is not None:
            elems = [int(v) for v in np.asarray(f.data(pl)).ravel()]
        else:
            raise CgnsError(f"boundary condition {bc.name!r} without a point "
                            "set")
        pts = []
        for e in elems:
            pts.extend(eind[eptr[e - 1]:eptr[e]].tolist())
        patches[bc.name] = pts
    # cells: the elements with more than two nodes, in element-id order
    sizes = np.diff(eptr)
    keep = np.nonzero(sizes > 2)[0]
    cptr = np.zeros(keep.size + 1, np.int64)
    cptr[1:] = np.cumsum(sizes[keep])
    cind = np.concatenate([eind[eptr[e]:eptr[e + 1]] for e in keep]) \
        if keep.size else np.zeros(0, np.int64)
    return dict(nodes=nodes, cptr=cptr, cind=cind.astype(np.int64),
                patches=patches, base=base.name, zone=zone.name,
                n_elements=n_elem)


def patch_of_faces(nodes, patches, face_x, face_y, rcell):
    """Patch index of every face (-1 interior or unassigned) and the patch
    names, from the patches' node pairs (createPatchByNodes): a face's
    centroid is the midpoint of its two nodes (Face.cpp:9-18), so each pair
    is matched to the boundary face with that centroid.  A face listed by
    two patches belongs to the later one, as createPatchByNodes keeps the
    last registration."""
    names = sorted(patches)
    bf = np.nonzero(np.asarray(rcell) < 0)[0]
    key = {(float(face_x[f]), float(face_y[f])): int(f) for f in bf}
    out = np.full(len(face_x), -1, np.int32)
    for pi, name in enumerate(names):
        pts = patches[name]
        for a, b in zip(pts[0::2], pts[1::2]):
            mx = 0.5 * (nodes[a, 0] + nodes[b, 0])
            my = 0.5 * (nodes[a, 1] + nodes[b, 1])
            f = key.get((float(mx), float(my)))
            if f is None:
                raise CgnsError(f"patch {name!r}: nodes {a}, {b} are not a "
                                "boundary face")
            out[f] = pi
    return out, names
