"""ctypes binding of the scene/stepping facade.

The product library exports the facade with the ``vx_`` prefix (``include/vx_capi.h``); test
infrastructure exports the same function list under other prefixes, so :class:`Sim` takes the
library path and the prefix.  Each method mirrors one call of the reference's public C++ API
(``CVoxelyze`` in Voxelyze.h, ``CVX_Material`` in VX_Material.h, ``CVX_External`` in
VX_External.h, ``CVX_Voxel`` in VX_Voxel.h) with the same argument meaning and error behaviour:
setters return False where the reference returns false, ``do_time_step`` returns False on
divergence (Voxelyze.cpp:265-269).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

# material property ids (VX_Material.h:75-107)
PROP_POISSON, PROP_CTE, PROP_MU_STATIC, PROP_MU_KINETIC = 0, 1, 2, 3
PROP_ZETA_INTERNAL, PROP_ZETA_GLOBAL, PROP_ZETA_COLLISION, PROP_DENSITY = 4, 5, 6, 7

# dofComponent bits (VX_External.h:18-25)
X_TRANSLATE, Y_TRANSLATE, Z_TRANSLATE = 1, 2, 4
X_ROTATE, Y_ROTATE, Z_ROTATE = 8, 16, 32

# stateInfoType / valueType (Voxelyze.h:48-67)
(DISPLACEMENT, VELOCITY, KINETIC_ENERGY, ANGULAR_DISPLACEMENT, ANGULAR_VELOCITY, ENG_STRESS,
 ENG_STRAIN, STRAIN_ENERGY, PRESSURE, MASS) = range(10)
MIN, MAX, TOTAL, AVERAGE = range(4)

_d = C.c_double
_f = C.c_float
_i = C.c_int
_p = C.c_void_p
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)

_SIGS = {
    "create": (_p, [_d]),
    "remove_voxel": (_i, [_p, _i, _i, _i]),
    "replace_material": (_i, [_p, _i, _i]),
    "remove_material": (_i, [_p, _i]),
    "set_voxel_size": (None, [_p, _d]),
    "destroy": (None, [_p]),
    "add_material": (_i, [_p, _f, _f]),
    "material_set": (_i, [_p, _i, _i, _f]),
    "material_set_model_linear": (_i, [_p, _i, _f, _f]),
    "material_set_model_bilinear": (_i, [_p, _i, _f, _f, _f, _f]),
    "material_set_model": (_i, [_p, _i, _i, _fp, _fp]),
    "set_voxel": (_i, [_p, _i, _i, _i, _i]),
    "set_voxels": (_i, [_p, _i, _ip, _ip]),
    "voxel_count": (_i, [_p]),
    "link_count": (_i, [_p]),
    "voxel_index": (_i, [_p, _i, _i, _i]),
    "external_set_fixed": (_i, [_p, _i, _i]),
    "external_set_fixed_all": (_i, [_p, _i, _i]),
    "external_set_displacement": (_i, [_p, _i, _i, _d]),
    "external_set_displacement_all": (_i, [_p, _i, _dp, _dp]),
    "external_clear_displacement": (_i, [_p, _i, _i]),
    "external_set_force": (_i, [_p, _i, _f, _f, _f]),
    "external_set_moment": (_i, [_p, _i, _f, _f, _f]),
    "set_gravity": (None, [_p, _f]),
    "enable_floor": (None, [_p, _i]),
    "enable_collisions": (None, [_p, _i]),
    "set_ambient_temperature": (None, [_p, _f, _i]),
    "voxel_set_temperature": (_i, [_p, _i, _f]),
    "do_time_step": (_i, [_p, _f]),
    "do_time_steps": (_i, [_p, _i, _f]),
    "recommended_time_step": (_f, [_p]),
    "reset_time": (None, [_p]),
    "current_time": (_f, [_p]),
    "get_voxel_state": (_i, [_p, _dp, _fp, _ip]),
    "get_link_state": (_i, [_p, _dp, _fp, _ip]),
    "get_collisions": (_i, [_p, _ip, _i]),
    "state_info": (_f, [_p, _i, _i]),
    "voxel_external_force": (_i, [_p, _i, _fp]),
    "voxel_external_moment": (_i, [_p, _i, _fp]),
    "voxel_corner_offset": (_i, [_p, _i, _i, _fp]),
    "voxel_corner_position": (_i, [_p, _i, _i, _fp]),
    "voxel_force": (_i, [_p, _i, _dp]),
    "voxel_moment": (_i, [_p, _i, _dp]),
    "voxel_is_yielded": (_i, [_p, _i]),
    "voxel_is_failed": (_i, [_p, _i]),
    "voxel_pressure": (_f, [_p, _i]),
    "link_strain_energy": (_f, [_p, _i]),
    "link_is_yielded": (_i, [_p, _i]),
    "link_is_failed": (_i, [_p, _i]),
}


# scene-file entry points: in the product and the reference build, not in the oracle
_OPT_SIGS = {
    "material_stress": (_f, [_p, _i, _f, _f, _i]),
    "material_modulus": (_f, [_p, _i, _f]),
    "load_json": (_i, [_p, C.c_char_p]),
    "save_json": (_i, [_p, C.c_char_p]),
    "mesh_generate": (_i, [_p]),
    "mesh_update": (_i, [_p, _i, _i]),
    "mesh_counts": (_i, [_p, _ip]),
    "mesh_read": (_i, [_p, _fp, _ip, _fp, _fp, _ip]),
    "mesh_save_obj": (_i, [_p, C.c_char_p]),
}

# CVX_MeshRender::viewColoring
MESH_MATERIAL, MESH_FAILURE, MESH_STATE_INFO = 0, 1, 2


def bind(lib: C.CDLL, prefix: str) -> dict:
    """Resolve every facade symbol ``<prefix>_<name>`` in ``lib`` and set its ctypes signature."""
    fns = {}
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, f"{prefix}_{name}")
        fn.restype = res
        fn.argtypes = args
        fns[name] = fn
    for name, (res, args) in _OPT_SIGS.items():
        fn = getattr(lib, f"{prefix}_{name}", None)
        if fn is not None:
            fn.restype = res
            fn.argtypes = args
            fns[name] = fn
    return fns


def _ptr(a: Optional[np.ndarray], ct):
    return None if a is None else a.ctypes.data_as(C.POINTER(ct))


class Sim:
    """One simulation instance (one ``CVoxelyze``) behind a facade library."""

    def __init__(self, lib: C.CDLL, prefix: str, voxel_size: float = 0.001, fns: dict | None = None):
        self.lib = lib
        self.prefix = prefix
        self.f = fns if fns is not None else bind(lib, prefix)
        self.h = self.f["create"](voxel_size)
        if not self.h:
            raise RuntimeError(f"{prefix}_create failed")

    def close(self):
        if self.h:
            self.f["destroy"](self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- materials -------------------------------------------------------------------------
    def add_material(self, E: float = 1e6, rho: float = 1e3) -> int:
        return self.f["add_material"](self.h, E, rho)

    def material_set(self, mat: int, prop: int, value: float) -> bool:
        return self.f["material_set"](self.h, mat, prop, value) == 0

    def set_model_linear(self, mat, E, fail=-1.0) -> bool:
        return self.f["material_set_model_linear"](self.h, mat, E, fail) == 0

    def set_model_bilinear(self, mat, E, plastic_E, yield_stress, fail=-1.0) -> bool:
        return self.f["material_set_model_bilinear"](self.h, mat, E, plastic_E, yield_stress, fail) == 0

    def set_model(self, mat, strain, stress) -> bool:
        a = np.ascontiguousarray(strain, dtype=np.float32)
        b = np.ascontiguousarray(stress, dtype=np.float32)
        return self.f["material_set_model"](self.h, mat, len(a), _ptr(a, C.c_float), _ptr(b, C.c_float)) == 0

    def material_stress(self, mat, strain, tss=0.0, force_linear=False) -> float:
        """CVX_Material::stress (src/VX_Material.cpp:165-195)."""
        return self.f["material_stress"](self.h, mat, strain, tss, 1 if force_linear else 0)

    def material_modulus(self, mat, strain) -> float:
        """CVX_Material::modulus (src/VX_Material.cpp:214-226)."""
        return self.f["material_modulus"](self.h, mat, strain)

    # -- voxels ----------------------------------------------------------------------------
    def set_voxel(self, mat: int, x: int, y: int, z: int) -> int:
        return self.f["set_voxel"](self.h, mat, x, y, z)

    def set_voxels(self, mats: np.ndarray, xyz: np.ndarray) -> None:
        m = np.ascontiguousarray(mats, dtype=np.int32)
        p = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1)
        self.f["set_voxels"](self.h, len(m), _ptr(m, C.c_int), _ptr(p, C.c_int))

    def voxel_count(self) -> int:
        return self.f["voxel_count"](self.h)

    def link_count(self) -> int:
        return self.f["link_count"](self.h)

    def voxel_index(self, x, y, z) -> int:
        return self.f["voxel_index"](self.h, x, y, z)

    # -- externals -------------------------------------------------------------------------
    def set_fixed(self, v, mask: int):
        self.f["external_set_fixed"](self.h, v, mask)

    def set_fixed_all(self, v, fixed=True):
        self.f["external_set_fixed_all"](self.h, v, 1 if fixed else 0)

    def set_displacement(self, v, dof: int, value: float = 0.0):
        self.f["external_set_displacement"](self.h, v, dof, value)

    def set_displacement_all(self, v, translation=(0.0, 0.0, 0.0), rotation=(0.0, 0.0, 0.0)):
        t = np.ascontiguousarray(translation, dtype=np.float64)
        r = np.ascontiguousarray(rotation, dtype=np.float64)
        self.f["external_set_displacement_all"](self.h, v, _ptr(t, C.c_double), _ptr(r, C.c_double))

    def clear_displacement(self, v, dof: int):
        self.f["external_clear_displacement"](self.h, v, dof)

    def set_force(self, v, fx, fy, fz):
        self.f["external_set_force"](self.h, v, fx, fy, fz)

    def set_moment(self, v, mx, my, mz):
        self.f["external_set_moment"](self.h, v, mx, my, mz)

    # -- globals ---------------------------------------------------------------------------
    def set_gravity(self, g: float = 1.0):
        self.f["set_gravity"](self.h, g)

    def enable_floor(self, on=True):
        self.f["enable_floor"](self.h, 1 if on else 0)

    def enable_collisions(self, on=True):
        self.f["enable_collisions"](self.h, 1 if on else 0)

    def set_ambient_temperature(self, t: float, all_voxels: bool = False):
        self.f["set_ambient_temperature"](self.h, t, 1 if all_voxels else 0)

    def set_temperature(self, v: int, t: float):
        self.f["voxel_set_temperature"](self.h, v, t)

    # -- stepping --------------------------------------------------------------------------
    def do_time_step(self, dt: float = -1.0) -> bool:
        return self.f["do_time_step"](self.h, dt) == 1

    def do_time_steps(self, n: int, dt: float = -1.0) -> int:
        return self.f["do_time_steps"](self.h, n, dt)

    def recommended_time_step(self) -> float:
        return self.f["recommended_time_step"](self.h)

    def reset_time(self):
        self.f["reset_time"](self.h)

    # -- topology edits (CVoxelyze::setVoxel(NULL), replaceMaterial, removeMaterial,
    #    setVoxelSize) ---------------------------------------------------------------------
    def remove_voxel(self, x: int, y: int, z: int):
        self.f["remove_voxel"](self.h, x, y, z)

    def replace_material(self, a: int, b: int) -> bool:
        return self.f["replace_material"](self.h, a, b) == 0

    def remove_material(self, m: int) -> bool:
        return self.f["remove_material"](self.h, m) == 0

    def set_voxel_size(self, size: float):
        self.f["set_voxel_size"](self.h, size)

    # -- scene files (CVoxelyze::loadJSON / saveJSON) ---------------------------------------
    def load_json(self, path: str) -> bool:
        return self.f["load_json"](self.h, path.encode()) == 1

    def save_json(self, path: str) -> bool:
        return self.f["save_json"](self.h, path.encode()) == 1

    # -- deformed mesh (CVX_MeshRender) -----------------------------------------------------
    def mesh_generate(self) -> bool:
        """Builds (or rebuilds) the mesh and updates it once; False if the update could not run."""
        return self.f["mesh_generate"](self.h) == 0

    def mesh_update(self, coloring: int = 0, state_info: int = 0) -> bool:
        return self.f["mesh_update"](self.h, coloring, state_info) == 0

    def mesh(self) -> dict:
        n = np.zeros(3, np.int32)
        if self.f["mesh_counts"](self.h, _ptr(n, C.c_int)) != 0:
            raise RuntimeError("no mesh: call mesh_generate first")
        nv, nq, nl = (int(x) for x in n)
        out = {"vertices": np.zeros((nv, 3), np.float32), "quads": np.zeros((nq, 4), np.int32),
               "normals": np.zeros((nq, 3), np.float32), "colors": np.zeros((nq, 3), np.float32),
               "lines": np.zeros((nl, 2), np.int32)}
        self.f["mesh_read"](self.h, _ptr(out["vertices"], C.c_float), _ptr(out["quads"], C.c_int),
                            _ptr(out["normals"], C.c_float), _ptr(out["colors"], C.c_float),
                            _ptr(out["lines"], C.c_int))
        return out

    def mesh_save_obj(self, path: str) -> bool:
        return self.f["mesh_save_obj"](self.h, path.encode()) == 0

    def current_time(self) -> float:
        return self.f["current_time"](self.h)

    def state_info(self, info: int, vtype: int) -> float:
        return self.f["state_info"](self.h, info, vtype)

    # -- per-voxel and per-link queries (VX_Voxel.h:79-130, VX_Link.h:47-66) -----------------
    def _vec(self, name, ct, *args) -> np.ndarray:
        out = np.zeros(3, np.float32 if ct is C.c_float else np.float64)
        if self.f[name](self.h, *args, _ptr(out, ct)) != 0:
            raise IndexError(f"{name}{args}")
        return out

    def external_force(self, v: int) -> np.ndarray:
        """CVX_Voxel::externalForce: applied force, reaction force on fixed translations."""
        return self._vec("voxel_external_force", C.c_float, v)

    def external_moment(self, v: int) -> np.ndarray:
        return self._vec("voxel_external_moment", C.c_float, v)

    def corner_offset(self, v: int, corner: int) -> np.ndarray:
        return self._vec("voxel_corner_offset", C.c_float, v, corner)

    def corner_position(self, v: int, corner: int) -> np.ndarray:
        return self._vec("voxel_corner_position", C.c_float, v, corner)

    def voxel_force(self, v: int) -> np.ndarray:
        return self._vec("voxel_force", C.c_double, v)

    def voxel_moment(self, v: int) -> np.ndarray:
        return self._vec("voxel_moment", C.c_double, v)

    def voxel_is_yielded(self, v: int) -> bool:
        return self.f["voxel_is_yielded"](self.h, v) == 1

    def voxel_is_failed(self, v: int) -> bool:
        return self.f["voxel_is_failed"](self.h, v) == 1

    def pressure(self, v: int) -> float:
        return self.f["voxel_pressure"](self.h, v)

    def strain_energy(self, l: int) -> float:
        return self.f["link_strain_energy"](self.h, l)

    def link_is_yielded(self, l: int) -> bool:
        return self.f["link_is_yielded"](self.h, l) == 1

    def link_is_failed(self, l: int) -> bool:
        return self.f["link_is_failed"](self.h, l) == 1

    def queries(self, corners=range(8)) -> dict:
        """Every per-voxel and per-link query for the whole scene, as arrays (for comparisons)."""
        nv, nl = self.voxel_count(), self.link_count()
        return {
            "external_force": np.array([self.external_force(v) for v in range(nv)]).reshape(nv, 3),
            "external_moment": np.array([self.external_moment(v) for v in range(nv)]).reshape(nv, 3),
            "corner_offset": np.array([[self.corner_offset(v, c) for c in corners] for v in range(nv)]),
            "corner_position": np.array([[self.corner_position(v, c) for c in corners] for v in range(nv)]),
            "voxel_yielded": np.array([self.voxel_is_yielded(v) for v in range(nv)]),
            "voxel_failed": np.array([self.voxel_is_failed(v) for v in range(nv)]),
            "pressure": np.array([self.pressure(v) for v in range(nv)], np.float32),
            "strain_energy": np.array([self.strain_energy(l) for l in range(nl)], np.float32),
            "link_yielded": np.array([self.link_is_yielded(l) for l in range(nl)]),
            "link_failed": np.array([self.link_is_failed(l) for l in range(nl)]),
            "force": np.array([self.voxel_force(v) for v in range(nv)]).reshape(nv, 3),
            "moment": np.array([self.voxel_moment(v) for v in range(nv)]).reshape(nv, 3),
        }

    # -- readback --------------------------------------------------------------------------
    def voxel_state(self) -> dict:
        n = self.voxel_count()
        d = np.zeros((n, 13), np.float64)
        f = np.zeros((n, 5), np.float32)
        i = np.zeros((n, 2), np.int32)
        self.f["get_voxel_state"](self.h, _ptr(d, C.c_double), _ptr(f, C.c_float), _ptr(i, C.c_int))
        return {"pos": d[:, 0:3], "linMom": d[:, 3:6], "orient": d[:, 6:10], "angMom": d[:, 10:13],
                "temp": f[:, 0], "previousDt": f[:, 1], "pStrain": f[:, 2:5],
                "staticFriction": i[:, 0], "pStrainInvalid": i[:, 1], "raw_d": d, "raw_f": f, "raw_i": i}

    def link_state(self) -> dict:
        n = self.link_count()
        d = np.zeros((n, 22), np.float64)
        f = np.zeros((n, 6), np.float32)
        i = np.zeros((n, 6), np.int32)
        self.f["get_link_state"](self.h, _ptr(d, C.c_double), _ptr(f, C.c_float), _ptr(i, C.c_int))
        return {"pos2": d[:, 0:3], "angle1v": d[:, 3:6], "angle2v": d[:, 6:9], "forceNeg": d[:, 9:12],
                "forcePos": d[:, 12:15], "momentNeg": d[:, 15:18], "momentPos": d[:, 18:21],
                "restLength": d[:, 21], "strain": f[:, 0], "maxStrain": f[:, 1], "strainOffset": f[:, 2],
                "stress": f[:, 3], "transverseArea": f[:, 4], "transverseStrainSum": f[:, 5],
                "smallAngle": i[:, 0], "localVelValid": i[:, 1], "axis": i[:, 2], "vneg": i[:, 3],
                "vpos": i[:, 4], "mat": i[:, 5], "raw_d": d, "raw_f": f, "raw_i": i}

    def collisions(self) -> np.ndarray:
        n = self.f["get_collisions"](self.h, None, 0)
        out = np.zeros((max(n, 1), 2), np.int32)
        self.f["get_collisions"](self.h, _ptr(out, C.c_int), n)
        return out[:n]


# -- product extensions (include/vx_capi.h, "extensions for throughput users") --------------------
_EXT_SIGS = {
    "set_precision": (_i, [_p, _i]),
    "read_positions": (_i, [_p, _dp]),
    "read_positions_async": (_i, [_p, _dp]),
    "read_wait": (_i, [_p]),
    "set_temperatures": (_i, [_p, _fp]),
    "state_info_device": (_f, [_p, _i, _i]),
    "counters": (_i, [_p, C.POINTER(C.c_longlong), _i]),
    "enable_timing": (_i, [_p, _i]),
    "step_timing": (_i, [_p, _fp]),
    "last_error": (C.c_char_p, [_p]),
    "set_actuation": (_i, [_p, _i, _d, _d, _fp]),
    "body_com": (_i, [_p, _ip, _i, _dp]),
    "snapshot": (_i, [_p, _i]),
    "restore": (_i, [_p, _i]),
    "set_launch": (_i, [_p, _i, _i, _i]),
    "autotune": (_i, [_p, _i, _f, _ip]),
    "get_launch": (_i, [_p, _ip, _ip, _ip]),
    "set_link_pipeline": (_i, [_p, _i]),
    "get_link_pipeline": (_i, [_p, _ip]),
    "set_link_split": (_i, [_p, _i]),
    "set_body_batches": (_i, [_p, _i]),
    "get_body_batches": (_i, [_p, _ip, _ip]),
    "get_link_split": (_i, [_p, _ip]),
    "set_decisions": (_i, [_p, _i, C.c_longlong]),
    "get_decisions": (_i, [_p, C.POINTER(C.c_ubyte), C.c_longlong]),
    "put_decisions": (_i, [_p, C.POINTER(C.c_ubyte), C.c_longlong]),
    "set_poisson_fusion": (_i, [_p, _i]),
    "adjoint_com_x": (_i, [_p, _i, _f, _i, _ip, _i, _dp, _dp, _dp, _dp]),
}

ACT_OFF, ACT_UNIFORM, ACT_PER_VOXEL = 0, 1, 2


class Engine:
    """The product library's extensions on one :class:`Sim` (prefix ``vx``): precision mode,
    per-step actuation, body centres of mass, device snapshots and launch tuning."""

    def __init__(self, sim: Sim):
        if sim.prefix != "vx":
            raise ValueError("engine extensions exist on the product library only")
        self.sim = sim
        self.f = {}
        for name, (res, args) in _EXT_SIGS.items():
            fn = getattr(sim.lib, f"vx_{name}")
            fn.restype = res
            fn.argtypes = args
            self.f[name] = fn

    def _ck(self, rc):
        if rc != 0:
            raise RuntimeError(self.f["last_error"](self.sim.h).decode(errors="replace") or f"error {rc}")

    def set_precision(self, mode: int):
        self._ck(self.f["set_precision"](self.sim.h, mode))

    def set_actuation(self, mode: int, amplitude: float = 0.0, frequency: float = 0.0, phase=None):
        ph = None if phase is None else np.ascontiguousarray(phase, np.float32)
        self._ck(self.f["set_actuation"](self.sim.h, mode, amplitude, frequency, _ptr(ph, C.c_float)))

    def body_com(self, offsets) -> np.ndarray:
        off = np.ascontiguousarray(offsets, np.int32)
        out = np.zeros((len(off) - 1, 3), np.float64)
        self._ck(self.f["body_com"](self.sim.h, _ptr(off, C.c_int), len(off) - 1, _ptr(out, C.c_double)))
        return out

    def snapshot(self, slot: int = 0):
        self._ck(self.f["snapshot"](self.sim.h, slot))

    def restore(self, slot: int = 0):
        self._ck(self.f["restore"](self.sim.h, slot))

    def set_launch(self, block_link: int = 0, block_voxel: int = 0, graph_chunk: int = 0):
        self._ck(self.f["set_launch"](self.sim.h, block_link, block_voxel, graph_chunk))

    def set_link_pipeline(self, blocks_per_sm: int):
        """FP32C link pass: >0 pipelined kernel with that many resident blocks per SM, -1 as many
        as fit, 0 the one-thread-per-link kernel (default)."""
        self._ck(self.f["set_link_pipeline"](self.sim.h, blocks_per_sm))

    def set_link_split(self, on: bool):
        """FP32C link pass at a fixed dt: the small-angle kernel plus the general kernel over the
        links it defers, or the general kernel over every link (default); identical results."""
        self._ck(self.f["set_link_split"](self.sim.h, 1 if on else 0))

    def set_body_batches(self, voxels_per_group: int):
        """FP32C, fixed dt, no collisions, bodies no link joins: each batch in one persistent launch
        whose CTAs run groups of bodies (up to voxels_per_group voxels; 1: one body per group;
        0: off) through every step; identical results."""
        self._ck(self.f["set_body_batches"](self.sim.h, int(voxels_per_group)))

    def body_batches(self) -> tuple[int, int]:
        """(voxels per group, groups of the current scene)."""
        out = np.zeros(2, np.int32)
        self._ck(self.f["get_body_batches"](self.sim.h, _ptr(out[:1], C.c_int), _ptr(out[1:], C.c_int)))
        return int(out[0]), int(out[1])

    def link_split(self) -> bool:
        out = np.zeros(1, np.int32)
        self._ck(self.f["get_link_split"](self.sim.h, _ptr(out, C.c_int)))
        return bool(out[0])

    def set_poisson_fusion(self, on: bool):
        """FP32C, nu != 0: fill the Poisson-strain cache in the voxel pass (default) or in a
        pre-pass before every link pass; the trajectories are identical."""
        self._ck(self.f["set_poisson_fusion"](self.sim.h, 1 if on else 0))

    def set_decisions(self, mode: int, steps: int = 0):
        """FP64: 1 records the floor-contact and static-friction decisions of the next `steps`
        steps (one byte per voxel per step), 2 replays them, 0 stops."""
        self._ck(self.f["set_decisions"](self.sim.h, mode, steps))

    def decisions(self, steps: int) -> np.ndarray:
        out = np.zeros((steps, self.sim.voxel_count()), np.uint8)
        self._ck(self.f["get_decisions"](self.sim.h, _ptr(out, C.c_ubyte), steps))
        return out

    def put_decisions(self, rows: np.ndarray):
        rows = np.ascontiguousarray(rows, np.uint8)
        self._ck(self.f["put_decisions"](self.sim.h, _ptr(rows, C.c_ubyte), rows.shape[0]))

    def link_pipeline(self) -> int:
        out = np.zeros(1, np.int32)
        self._ck(self.f["get_link_pipeline"](self.sim.h, _ptr(out, C.c_int)))
        return int(out[0])

    def launch(self) -> tuple:
        """(threads per block of the link pass, of the voxel pass, steps per captured graph)."""
        out = np.zeros(3, np.int32)
        self._ck(self.f["get_launch"](self.sim.h, _ptr(out[0:], C.c_int), _ptr(out[1:], C.c_int),
                                      _ptr(out[2:], C.c_int)))
        return tuple(int(x) for x in out)

    def autotune(self, trial_steps: int = 20, dt: float = -1.0) -> tuple:
        out = np.zeros(3, np.int32)
        self._ck(self.f["autotune"](self.sim.h, trial_steps, dt, _ptr(out, C.c_int)))
        return tuple(int(x) for x in out)

    def adjoint_com_x(self, nsteps: int, dt: float, body_offsets, checkpoint_every: int = 100):
        """Run nsteps from the current state; return (per-body centre-of-mass x after the run,
        dJ/dE, dJ/drho, dJ/dphase per voxel) for J = the sum of the per-body values."""
        off = np.ascontiguousarray(body_offsets, np.int32)
        nb, nv = len(off) - 1, self.sim.voxel_count()
        obj = np.zeros(nb, np.float64)
        gE, gR, gP = (np.zeros(nv, np.float64) for _ in range(3))
        self._ck(self.f["adjoint_com_x"](self.sim.h, nsteps, dt, checkpoint_every, _ptr(off, C.c_int), nb,
                                         _ptr(obj, C.c_double), _ptr(gE, C.c_double), _ptr(gR, C.c_double),
                                         _ptr(gP, C.c_double)))
        return obj, gE, gR, gP

    def read_positions(self) -> np.ndarray:
        n = self.sim.voxel_count()
        out = np.zeros(3 * n, np.float64)
        self._ck(self.f["read_positions"](self.sim.h, _ptr(out, C.c_double)))
        return out.reshape(3, n).T

    def read_positions_async(self, out: np.ndarray):
        """Start copying every voxel's position into ``out`` (3 n float64, component-major) while
        later steps run; ``out`` holds them once read_wait() returns.  The copy overlaps only for
        pinned memory (a numpy array waits for it)."""
        if out.dtype != np.float64 or out.size != 3 * self.sim.voxel_count() or not out.flags.c_contiguous:
            raise ValueError("needs a contiguous float64 array of 3 * voxel_count() elements")
        self._ck(self.f["read_positions_async"](self.sim.h, _ptr(out, C.c_double)))

    def read_wait(self):
        self._ck(self.f["read_wait"](self.sim.h))
