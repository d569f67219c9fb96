"""Python front end of libgpugi_bvhmake.so (the bvhmake restatement).

`build_bvh` returns the arrays in the layout the traversal kernels and the
file format use: `hierarchy` float32 [N, 8] (min.xyz, firstChild bits,
max.xyz, escape bits), `slots` int32 [S, 4] with leaf_size slots per block.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_LIB = None
LIB_DIR = Path(__file__).resolve().parent / "lib"

BUILD_METHODS = {"kdtree": 0, "sweep": 1, "lds": 2}
FIT_METHODS = {"aabox": 0, "ellipsoid": 1, "obox": 2}


def _lib():
    global _LIB
    if _LIB is None:
        path = LIB_DIR / "libgpugi_bvhmake.so"
        if not path.exists():
            raise RuntimeError(f"{path} is missing: run `python -m gpugi_gb300.build` first")
        lib = C.CDLL(str(path))
        P, U32, U64, I = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
        lib.gpugi_bvh_build.argtypes = [P, U32, P, U32, U32, U32, U32, U64, C.POINTER(P)]
        lib.gpugi_bvh_build.restype = I
        lib.gpugi_bvh_info.argtypes = [P] + [C.POINTER(U32)] * 5
        lib.gpugi_bvh_export.argtypes = [P, P, P, P]
        lib.gpugi_bvh_write_file.argtypes = [P, C.c_char_p]
        lib.gpugi_bvh_read_file.argtypes = [C.c_char_p, C.POINTER(P)]
        lib.gpugi_bvh_vertices.argtypes = [P, C.POINTER(U32), P]
        lib.gpugi_bvh_set_vertex_attributes.argtypes = [P, P, P]
        lib.gpugi_bvh_vertex_attributes.argtypes = [P, P, P]
        lib.gpugi_bvh_set_materials.argtypes = [P, P, U32]
        lib.gpugi_bvh_materials.argtypes = [P, C.POINTER(U32), P]
        lib.gpugi_bvh_set_material_names.argtypes = [P, P, U32]
        lib.gpugi_bvh_material_name.argtypes = [P, U32]
        lib.gpugi_bvh_material_name.restype = C.c_char_p
        lib.gpugi_bvh_num_material_names.argtypes = [P]
        lib.gpugi_bvh_num_material_names.restype = U32
        lib.gpugi_materials_from_json.argtypes = [C.c_char_p, P, U32, P]
        lib.gpugi_materials_from_json.restype = I
        lib.gpugi_materials_json_error.restype = C.c_char_p
        lib.gpugi_bvh_sggx.argtypes = [P, P]
        lib.gpugi_bvh_sggx.restype = I
        lib.gpugi_bvh_free.argtypes = [P]
        lib.gpugi_bvh_free.restype = None
        lib.gpugi_bvh_last_error.restype = C.c_char_p
        _LIB = lib
    return _LIB


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


@dataclass
class BVH:
    hierarchy: np.ndarray   # float32 [N, 8] ([N, 12] for oriented boxes: + rotationInv quaternion)
    slots: np.ndarray       # int32 [S, 4]
    parents: np.ndarray     # uint32 [N]
    leaf_size: int
    bounds_kind: int        # 0 = AABB, 1 = ellipsoid, 2 = oriented box
    max_depth: int
    positions: np.ndarray | None = None
    normals: np.ndarray | None = None      # from a file: float32 [V, 3]
    texcoords: np.ndarray | None = None    # from a file: float32 [V, 2]
    materials: np.ndarray | None = None    # from a file: float32 [M, 24] (empty when absent)
    material_names: list | None = None     # from a file: the "materialref" chunk
    sggx: np.ndarray | None = None         # uint16 [N, 6] node NDFs {sigma.xyz, r.xyz} ("approx_sggx")

    @property
    def num_nodes(self) -> int:
        return self.hierarchy.shape[0]

    @property
    def num_slots(self) -> int:
        return self.slots.shape[0]

    @property
    def first_child(self) -> np.ndarray:
        return self.hierarchy[:, 3].view(np.uint32)

    @property
    def escape(self) -> np.ndarray:
        return self.hierarchy[:, 7].view(np.uint32)


def _collect(handle) -> BVH:
    lib = _lib()
    n, nb, ls, bk, md = (C.c_uint32() for _ in range(5))
    lib.gpugi_bvh_info(handle, C.byref(n), C.byref(nb), C.byref(ls), C.byref(bk), C.byref(md))
    hier = np.zeros((n.value, 12 if bk.value == 2 else 8), dtype=np.float32)
    slots = np.zeros((nb.value * ls.value, 4), dtype=np.int32)
    parents = np.zeros(n.value, dtype=np.uint32)
    lib.gpugi_bvh_export(handle, _ptr(hier), _ptr(slots), _ptr(parents))
    return BVH(hier, slots, parents, ls.value, bk.value, md.value)


def _sggx(lib, h, num_nodes) -> np.ndarray:
    out = np.zeros((num_nodes, 6), dtype=np.uint16)
    if lib.gpugi_bvh_sggx(h, _ptr(out)) != 0:
        raise ValueError(lib.gpugi_bvh_last_error().decode())
    return out


def build_bvh(positions: np.ndarray, triangles: np.ndarray, method: str = "sweep", fit: str = "aabox",
              leaf_size: int = 8, seed: int = 1, normals: np.ndarray | None = None) -> BVH:
    """Build the hierarchy; with per-vertex normals also the node NDFs
    (bvhmake's approx_sggx)."""
    lib = _lib()
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    tri = np.ascontiguousarray(triangles, dtype=np.uint32)
    h = C.c_void_p()
    rc = lib.gpugi_bvh_build(_ptr(pos), pos.shape[0], _ptr(tri), tri.shape[0], BUILD_METHODS[method],
                             FIT_METHODS[fit], leaf_size, seed, C.byref(h))
    if rc != 0:
        raise ValueError(f"gpugi_bvh_build failed ({rc}): {lib.gpugi_bvh_last_error().decode()}")
    try:
        b = _collect(h)
        b.positions = pos
        if normals is not None:
            nrm = np.ascontiguousarray(normals, dtype=np.float32)
            if nrm.shape != (pos.shape[0], 3):
                raise ValueError("normals need one row per vertex")
            lib.gpugi_bvh_set_vertex_attributes(h, _ptr(nrm), None)
            b.normals = nrm
            b.sggx = _sggx(lib, h, b.num_nodes)
        return b
    finally:
        lib.gpugi_bvh_free(h)


def _names_array(names):
    arr = (C.c_char_p * len(names))(*[n.encode() for n in names])
    return C.cast(arr, C.c_void_p), arr


def materials_from_json(text: str, names) -> np.ndarray:
    """Material records of the named materials of a gpugi scene JSON
    (Scene::LoadMaterial's mapping and defaults)."""
    lib = _lib()
    ptr, keep = _names_array(list(names))
    out = np.zeros((len(names), 24), dtype=np.float32)
    rc = lib.gpugi_materials_from_json(text.encode(), ptr, len(names), _ptr(out))
    if rc != 0:
        raise ValueError(lib.gpugi_materials_json_error().decode())
    return out


def write_bvh_file(positions: np.ndarray, triangles: np.ndarray, path: str, normals=None, texcoords=None,
                   materials=None, material_names=None, **kw) -> None:
    """Build and write bvhmake's NamedArray file (vertex normals/texcoords
    and material records are optional)."""
    lib = _lib()
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    tri = np.ascontiguousarray(triangles, dtype=np.uint32)
    h = C.c_void_p()
    rc = lib.gpugi_bvh_build(_ptr(pos), pos.shape[0], _ptr(tri), tri.shape[0],
                             BUILD_METHODS[kw.get("method", "sweep")], FIT_METHODS[kw.get("fit", "aabox")],
                             kw.get("leaf_size", 8), kw.get("seed", 1), C.byref(h))
    if rc != 0:
        raise ValueError(lib.gpugi_bvh_last_error().decode())
    try:
        nrm = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32)
        tc = None if texcoords is None else np.ascontiguousarray(texcoords, dtype=np.float32)
        for a, k in ((nrm, 3), (tc, 2)):
            if a is not None and a.shape != (pos.shape[0], k):
                raise ValueError("vertex attribute arrays need one row per vertex")
        lib.gpugi_bvh_set_vertex_attributes(h, None if nrm is None else _ptr(nrm), None if tc is None else _ptr(tc))
        if materials is not None:
            mats = np.ascontiguousarray(materials, dtype=np.float32).reshape(-1, 24)
            lib.gpugi_bvh_set_materials(h, _ptr(mats), mats.shape[0])
        if material_names is not None:
            ptr, keep = _names_array(list(material_names))
            if lib.gpugi_bvh_set_material_names(h, ptr, len(material_names)) != 0:
                raise ValueError(lib.gpugi_bvh_last_error().decode())
        if lib.gpugi_bvh_write_file(h, str(path).encode()) != 0:
            raise OSError(lib.gpugi_bvh_last_error().decode())
    finally:
        lib.gpugi_bvh_free(h)


def read_bvh_file(path: str) -> BVH:
    lib = _lib()
    h = C.c_void_p()
    if lib.gpugi_bvh_read_file(str(path).encode(), C.byref(h)) != 0:
        raise OSError(lib.gpugi_bvh_last_error().decode())
    try:
        b = _collect(h)
        nv = C.c_uint32()
        lib.gpugi_bvh_vertices(h, C.byref(nv), None)
        pos = np.zeros((nv.value, 3), dtype=np.float32)
        lib.gpugi_bvh_vertices(h, C.byref(nv), _ptr(pos))
        b.positions = pos
        b.normals = np.zeros((nv.value, 3), dtype=np.float32)
        b.texcoords = np.zeros((nv.value, 2), dtype=np.float32)
        lib.gpugi_bvh_vertex_attributes(h, _ptr(b.normals), _ptr(b.texcoords))
        nm = C.c_uint32()
        lib.gpugi_bvh_materials(h, C.byref(nm), None)
        b.materials = np.zeros((nm.value, 24), dtype=np.float32)
        if nm.value:
            lib.gpugi_bvh_materials(h, C.byref(nm), _ptr(b.materials))
        b.material_names = [lib.gpugi_bvh_material_name(h, i).decode()
                            for i in range(lib.gpugi_bvh_num_material_names(h))]
        # node NDFs: the file's approx_sggx chunk, else computed from the normals (when there are any)
        b.sggx = None
        if np.any(b.normals):
            try:
                b.sggx = _sggx(lib, h, b.num_nodes)
            except ValueError:
                b.sggx = None
        return b
    finally:
        lib.gpugi_bvh_free(h)
