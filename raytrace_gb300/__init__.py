"""GB300 renderer for the RayTracer per-pixel loop of XZiar/RayTrace.

Python view of the C ABI in include/rt_gb300.h (librt_gb300.so, loaded with ctypes). The
library holds the CUDA kernels; there is no CPU rendering path here: if the library is
missing, importing this package raises ImportError, and if no GPU is present the context
constructor raises RTError.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "librt_gb300.so")

RT_OK, RT_ERR_INVALID, RT_ERR_CUDA, RT_ERR_OOM, RT_ERR_CANCELLED = 0, -1, -2, -3, -4
RT_ERR_OVERFLOW, RT_ERR_TIMEOUT, RT_ERR_BUDGET, RT_ERR_NOT_FOUND, RT_ERR_BUSY = -5, -6, -7, -8, -9
RT_ERR_TOO_LARGE = -10
RT_NOALLOC_MAX_TRIS = 1 << 18
RT_OBJECT_SPHERE, RT_OBJECT_CUBE, RT_OBJECT_MODEL, RT_OBJECT_PLANE, RT_OBJECT_BALLPLANE = 1, 2, 3, 4, 5
RT_LIGHT_PARALLEL, RT_LIGHT_POINT, RT_LIGHT_SPOT = 1, 2, 3
RT_MODE_CHECK, RT_MODE_DEPTH, RT_MODE_NORMAL, RT_MODE_TEXTURE = 0x1, 0x2, 0x3, 0x4
RT_MODE_MATERIAL, RT_MODE_SHADOW, RT_MODE_REFLECT, RT_MODE_REFRACT, RT_MODE_RAYTRACE = 0x5, 0x6, 0x7, 0x8, 0x80
RT_FLAG_REF_TILES, RT_FLAG_HIT_PLANES, RT_FLAG_COUNT_WORK, RT_FLAG_PROFILE = 0x1, 0x2, 0x4, 0x8
RT_BUILD_RADIX, RT_BUILD_CLUSTER = 0, 1
KERNEL_KINDS = ("raygen", "extend", "shade", "shadow", "resolve", "other")

F3 = C.c_float * 3


class Camera(C.Structure):
    _fields_ = [("position", F3), ("u", F3), ("v", F3), ("n", F3), ("width", C.c_int32), ("height", C.c_int32),
                ("fovy", C.c_float), ("znear", C.c_float), ("zfar", C.c_float)]


class Light(C.Structure):
    _fields_ = [("type", C.c_int32), ("on", C.c_int32), ("position", F3), ("ambient", F3), ("diffuse", F3),
                ("specular", F3), ("attenuation", F3)]


class Material(C.Structure):
    _fields_ = [("ambient", F3), ("diffuse", F3), ("specular", F3), ("shininess", C.c_float),
                ("reflect", C.c_float), ("refract", C.c_float), ("rfr", C.c_float), ("texture", C.c_int32)]


class Texture(C.Structure):
    _fields_ = [("w", C.c_int32), ("h", C.c_int32), ("bgr", C.POINTER(C.c_uint8))]


class Object(C.Structure):
    _fields_ = [("type", C.c_int32), ("show", C.c_int32), ("material", C.c_int32), ("texture", C.c_int32),
                ("position", F3), ("radius", C.c_float), ("normal", F3), ("axisx", F3), ("axisy", F3),
                ("bmin", F3), ("bmax", F3), ("tri_first", C.c_int64), ("tri_count", C.c_int64)]


class SceneDesc(C.Structure):
    _fields_ = [("camera", Camera), ("env_light", F3),
                ("n_lights", C.c_int32), ("lights", C.POINTER(Light)),
                ("n_materials", C.c_int32), ("materials", C.POINTER(Material)),
                ("n_textures", C.c_int32), ("textures", C.POINTER(Texture)),
                ("n_objects", C.c_int32), ("objects", C.POINTER(Object)),
                ("n_tris", C.c_int64), ("tri_p", C.POINTER(C.c_float)), ("tri_n", C.POINTER(C.c_float)),
                ("tri_uv", C.POINTER(C.c_float)), ("tri_mtl", C.POINTER(C.c_int32)),
                ("tri_id", C.POINTER(C.c_int32))]


class RenderDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("max_level", C.c_int32),
                ("mode", C.c_int32), ("flags", C.c_int32), ("seed", C.c_uint64), ("camera", C.POINTER(Camera))]


class RenderStats(C.Structure):
    _fields_ = [("rays_primary", C.c_int64), ("rays_secondary", C.c_int64), ("rays_shadow", C.c_int64),
                ("nodes_visited", C.c_int64), ("tris_tested", C.c_int64), ("spheres_tested", C.c_int64),
                ("shadow_nodes_visited", C.c_int64), ("shadow_tris_tested", C.c_int64),
                ("shadow_spheres_tested", C.c_int64), ("ms", C.c_float), ("overflow_retries", C.c_int32),
                ("kernel_ms", C.c_float * 6), ("kernel_launches", C.c_int32 * 6), ("kernel_idle", C.c_float * 6)]

    def total_rays(self) -> int:
        return int(self.rays_primary + self.rays_secondary + self.rays_shadow)

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["kernel_ms"] = dict(zip(KERNEL_KINDS, list(self.kernel_ms)))
        d["kernel_launches"] = dict(zip(KERNEL_KINDS, list(self.kernel_launches)))
        d["kernel_idle"] = dict(zip(KERNEL_KINDS, list(self.kernel_idle)))
        return d


class BatchTuning(C.Structure):
    _fields_ = [("block", C.c_int32), ("tile", C.c_int32), ("stack", C.c_int32), ("use_graph", C.c_int32),
                ("min_blocks", C.c_int32), ("dynamic", C.c_int32), ("wave_rays", C.c_int64),
                ("shadow_chunk", C.c_int32), ("pixel_tile", C.c_int32), ("lanes", C.c_int32),
                ("reserved", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("max_inflight", C.c_int32), ("max_level", C.c_int32),
                ("spp", C.c_int32), ("plain", C.c_int32), ("queue_rays", C.c_int64), ("max_pixels", C.c_int64),
                ("keep_images", C.c_int32), ("stages", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("scene", C.c_int32), ("width", C.c_int32), ("height", C.c_int32), ("camera", Camera),
                ("seed", C.c_uint64), ("arrival_s", C.c_double)]


class RequestResult(C.Structure):
    _fields_ = [("request", C.c_int64), ("status", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("scene", C.c_int32), ("arrival_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double),
                ("samples", C.c_int64), ("rebuilt", C.c_int32), ("pad", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


class ServeStats(C.Structure):
    _fields_ = [("requests", C.c_int64), ("completed", C.c_int64), ("rejected", C.c_int64),
                ("evictions", C.c_int64), ("rebuilds", C.c_int64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_ms", C.c_double), ("max_ms", C.c_double), ("mrays_per_s", C.c_double),
                ("wall_s", C.c_double), ("rays", C.c_int64), ("peak_bytes", C.c_int64), ("waves", C.c_int64),
                ("mean_wave_requests", C.c_double), ("admitted_busy", C.c_int64), ("pixels", C.c_int64),
                ("wave_ms_mean", C.c_double), ("wave_ms_p50", C.c_double), ("wave_ms_p99", C.c_double),
                ("device_busy_s", C.c_double), ("host_step_s", C.c_double), ("host_wait_s", C.c_double),
                ("steps", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


P = C.c_void_p
_SIGS = {
    "rt_version": (C.c_int, []),
    "rt_ctx_create": (C.c_int, [C.c_int, C.POINTER(P)]),
    "rt_ctx_destroy": (None, [P]),
    "rt_last_error": (C.c_char_p, [P]),
    "rt_ctx_synchronize": (C.c_int, [P]),
    "rt_ctx_set_stream": (C.c_int, [P, P]),
    "rt_ctx_release_cached": (C.c_int, [P]),
    "rt_ctx_set_build": (C.c_int, [P, C.c_int32]),
    "rt_scene_upload": (C.c_int, [P, C.POINTER(SceneDesc), C.POINTER(C.c_int32)]),
    "rt_scene_update_camera": (C.c_int, [P, C.c_int32, C.POINTER(Camera)]),
    "rt_scene_rebuild": (C.c_int, [P, C.c_int32]),
    "rt_scene_release": (C.c_int, [P, C.c_int32]),
    "rt_scene_device_bytes": (C.c_int, [P, C.c_int32, C.POINTER(C.c_int64)]),
    "rt_scene_build_ms": (C.c_int, [P, C.c_int32, C.POINTER(C.c_float)]),
    "rt_frame_create": (C.c_int, [P, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]),
    "rt_frame_release": (C.c_int, [P, C.c_int32]),
    "rt_frame_download": (C.c_int, [P, C.c_int32, P, P, P, P, P]),
    "rt_frame_device_ptrs": (C.c_int, [P, C.c_int32, C.POINTER(P), C.POINTER(P)]),
    "rt_render": (C.c_int, [P, C.c_int32, C.c_int32, C.POINTER(RenderDesc)]),
    "rt_render_wait": (C.c_int, [P, C.POINTER(RenderStats)]),
    "rt_cancel": (C.c_int, [P]),
    "rt_poll": (C.c_int, [P]),
    "rt_render_host": (C.c_int, [P, C.POINTER(SceneDesc), C.POINTER(RenderDesc), P, P, C.POINTER(RenderStats)]),
    "rt_cancel_mark": (C.c_uint64, [P]),
    "rt_render_host_since": (C.c_int, [P, C.c_uint64, C.POINTER(SceneDesc), C.POINTER(RenderDesc), P, P,
                                       C.POINTER(RenderStats)]),
    "rt_ctx_set_tuning": (C.c_int, [P, C.POINTER(BatchTuning)]),
    "rt_ctx_get_tuning": (C.c_int, [P, C.POINTER(BatchTuning)]),
    "rt_batch_render": (C.c_int, [P, C.c_int32, P, P, P, C.POINTER(BatchTuning)]),
    "rt_batch_render_plain": (C.c_int, [P, C.c_int32, P, P, P]),
    "rt_batch_autotune": (C.c_int, [P, C.c_int32, P, P, P, C.POINTER(BatchTuning)]),
    "rt_server_create": (C.c_int, [P, C.POINTER(ServerConfig), C.POINTER(P)]),
    "rt_server_destroy": (None, [P]),
    "rt_selftest_conversions": (C.c_int, [P, P, C.c_int32, C.c_double, P, P, P]),
    "rt_server_last_error": (C.c_char_p, [P]),
    "rt_server_stats": (C.c_int, [P, C.POINTER(ServeStats)]),
    "rt_server_latencies": (C.c_int, [P, P, C.c_int64, C.POINTER(C.c_int64)]),
    "rt_server_wave_ms": (C.c_int, [P, P, C.c_int64, C.POINTER(C.c_int64)]),
    "rt_orbit_camera": (C.c_int, [C.POINTER(Camera), C.c_double, C.c_double, C.c_int32, C.c_int32,
                                  C.POINTER(Camera)]),
    "rt_server_add_scene": (C.c_int, [P, C.POINTER(SceneDesc), C.POINTER(C.c_int32)]),
    "rt_server_set_tuning": (C.c_int, [P, C.POINTER(BatchTuning)]),
    "rt_server_submit": (C.c_int, [P, C.POINTER(Request), C.POINTER(C.c_int64)]),
    "rt_server_step": (C.c_int, [P, C.POINTER(C.c_int32)]),
    "rt_server_drain": (C.c_int, [P]),
    "rt_server_result": (C.c_int, [P, C.c_int64, C.POINTER(RequestResult), P, P]),
    "rt_server_resident": (C.c_int, [P, C.c_int32, C.POINTER(C.c_int32)]),
    "rt_server_now": (C.c_double, [P]),
    "rt_server_run_poisson": (C.c_int, [P, C.c_double, C.c_double, C.c_uint64, C.POINTER(ServeStats)]),
    "rt_morton_sort": (C.c_int, [P, P, C.c_int64, P, P]),
    "rt_morton_sort_noalloc": (C.c_int, [P, C.c_int64, P, P, P]),
    "rt_scene_bvh_download": (C.c_int, [P, C.c_int32, P, P, C.POINTER(C.c_int64)]),
    "rt_scene_test_set_node_refs": (C.c_int, [P, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]),
    "rt_ctx_test_queue_entries": (C.c_int, [P, C.c_int64]),
    "rt_scenegen": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(P)]),
    "rt_scenegen_small": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.POINTER(P)]),
    "rt_scenegen_extras": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32, C.POINTER(P)]),
    "rt_scenegen_textured": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32, C.POINTER(P)]),
    "rt_scenegen_obj": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int32, C.c_int32, C.POINTER(P)]),
    "rt_scene_host_from_desc": (C.c_int, [C.POINTER(SceneDesc), C.c_int32, C.c_int32, C.c_uint64, C.POINTER(P)]),
    "rt_scene_host_desc": (C.POINTER(SceneDesc), [P]),
    "rt_scene_host_render_params": (C.c_int, [P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_uint64)]),
    "rt_scene_host_save": (C.c_int, [P, C.c_char_p]),
    "rt_scene_host_pin": (C.c_int, [P]),
    "rt_scene_host_bytes": (C.c_int64, [P]),
    "rt_scene_host_load": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "rt_scene_host_free": (None, [P]),
}


def _load() -> C.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


class RTError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"rt error {code}: {msg}")
        self.code = code


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(P)


class SceneHost:
    """A seeded scene held in host memory (flat rt_scene_desc + render parameters)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def config(cls, config: int, index: int = 0) -> "SceneHost":
        h = P()
        rc = lib.rt_scenegen(config, index, C.byref(h))
        if rc:
            raise RTError(rc, f"rt_scenegen({config}, {index})")
        return cls(h)

    @classmethod
    def small(cls, seed: int, n_spheres: int = 8, ico_freq: int = 0, width: int = 64, height: int = 64,
              refractive_every: int = 0) -> "SceneHost":
        h = P()
        rc = lib.rt_scenegen_small(seed, n_spheres, ico_freq, width, height, refractive_every, C.byref(h))
        if rc:
            raise RTError(rc, "rt_scenegen_small")
        return cls(h)

    @classmethod
    def extras(cls, seed: int, width: int = 128, height: int = 64) -> "SceneHost":
        h = P()
        rc = lib.rt_scenegen_extras(seed, width, height, C.byref(h))
        if rc:
            raise RTError(rc, "rt_scenegen_extras")
        return cls(h)

    @classmethod
    def textured(cls, seed: int, width: int = 128, height: int = 64) -> "SceneHost":
        """Checker-textured plane, a textured icosphere (planar uvs, procedural map), spheres, a cube."""
        h = P()
        rc = lib.rt_scenegen_textured(seed, width, height, C.byref(h))
        if rc:
            raise RTError(rc, "rt_scenegen_textured")
        return cls(h)

    @classmethod
    def from_obj(cls, obj_path: str, mtl_path: str, width: int = 128, height: int = 64) -> "SceneHost":
        """A model read by the drop-in OBJ/MTL loader (textures relative to the working directory)."""
        h = P()
        rc = lib.rt_scenegen_obj(obj_path.encode(), mtl_path.encode(), width, height, C.byref(h))
        if rc:
            raise RTError(rc, f"rt_scenegen_obj: cannot load {obj_path}")
        return cls(h)

    @classmethod
    def from_desc(cls, desc: SceneDesc, spp: int = 1, max_level: int = 3, seed: int = 0) -> "SceneHost":
        h = P()
        rc = lib.rt_scene_host_from_desc(C.byref(desc), spp, max_level, seed, C.byref(h))
        if rc:
            raise RTError(rc, "rt_scene_host_from_desc")
        return cls(h)

    def with_camera(self, width: int, height: int, spp: int | None = None, max_level: int | None = None,
                    seed: int | None = None) -> "SceneHost":
        """A copy of this scene rendered at another size (same camera basis and fov)."""
        d = SceneDesc.from_buffer_copy(self.desc)
        d.camera.width, d.camera.height = width, height
        s0, l0, e0 = self.params
        return SceneHost.from_desc(d, s0 if spp is None else spp, l0 if max_level is None else max_level,
                                   e0 if seed is None else seed)

    @classmethod
    def load(cls, path: str) -> "SceneHost":
        h = P()
        rc = lib.rt_scene_host_load(path.encode(), C.byref(h))
        if rc:
            raise RTError(rc, f"rt_scene_host_load({path})")
        return cls(h)

    def pin(self) -> None:
        rc = lib.rt_scene_host_pin(self._h)
        if rc:
            raise RTError(rc, "rt_scene_host_pin")

    @property
    def nbytes(self) -> int:
        return int(lib.rt_scene_host_bytes(self._h))

    def save(self, path: str) -> None:
        rc = lib.rt_scene_host_save(self._h, path.encode())
        if rc:
            raise RTError(rc, f"rt_scene_host_save({path})")

    @property
    def desc(self) -> SceneDesc:
        d = lib.rt_scene_host_desc(self._h).contents
        d._owner = self   # the view points into this object's memory: keep it alive
        return d

    def desc_ptr(self):
        return lib.rt_scene_host_desc(self._h)

    @property
    def params(self) -> tuple[int, int, int]:
        spp, lvl, seed = C.c_int32(), C.c_int32(), C.c_uint64()
        lib.rt_scene_host_render_params(self._h, C.byref(spp), C.byref(lvl), C.byref(seed))
        return spp.value, lvl.value, seed.value

    def tri_points(self) -> np.ndarray:
        d = self.desc
        n = d.n_tris
        if n == 0:
            return np.zeros((0, 9), np.float32)
        return np.ctypeslib.as_array(d.tri_p, shape=(n * 9,)).reshape(n, 9).copy()

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h and lib is not None:
            lib.rt_scene_host_free(h)


class Context:
    """One GPU context: scenes, frames and renders (rt_ctx)."""

    def __init__(self, device: int = 0):
        h = P()
        rc = lib.rt_ctx_create(device, C.byref(h))
        if rc:
            raise RTError(rc, "rt_ctx_create: no usable CUDA device" if rc == RT_ERR_CUDA else "rt_ctx_create")
        self._h = h

    @property
    def handle(self):
        return self._h

    def _ck(self, rc: int, what: str) -> None:
        if rc:
            raise RTError(rc, f"{what}: {lib.rt_last_error(self._h).decode(errors='replace')}")

    def upload(self, scene: SceneHost | SceneDesc) -> int:
        sid = C.c_int32()
        ptr = scene.desc_ptr() if isinstance(scene, SceneHost) else C.byref(scene)
        self._ck(lib.rt_scene_upload(self._h, ptr, C.byref(sid)), "rt_scene_upload")
        return sid.value

    def release_scene(self, sid: int) -> None:
        self._ck(lib.rt_scene_release(self._h, sid), "rt_scene_release")

    def rebuild(self, sid: int) -> float:
        self._ck(lib.rt_scene_rebuild(self._h, sid), "rt_scene_rebuild")
        ms = C.c_float()
        lib.rt_scene_build_ms(self._h, sid, C.byref(ms))
        return ms.value

    def device_bytes(self, sid: int) -> int:
        b = C.c_int64()
        self._ck(lib.rt_scene_device_bytes(self._h, sid, C.byref(b)), "rt_scene_device_bytes")
        return b.value

    def build_ms(self, sid: int) -> float:
        ms = C.c_float()
        self._ck(lib.rt_scene_build_ms(self._h, sid, C.byref(ms)), "rt_scene_build_ms")
        return ms.value

    def frame(self, w: int, h: int) -> int:
        fid = C.c_int32()
        self._ck(lib.rt_frame_create(self._h, w, h, C.byref(fid)), "rt_frame_create")
        return fid.value

    def release_frame(self, fid: int) -> None:
        self._ck(lib.rt_frame_release(self._h, fid), "rt_frame_release")

    @staticmethod
    def render_desc(width=0, height=0, spp=1, max_level=3, mode=RT_MODE_RAYTRACE, flags=0, seed=0,
                    camera: Camera | None = None) -> RenderDesc:
        rd = RenderDesc(width, height, spp, max_level, mode, flags, seed, None)
        if camera is not None:
            rd._cam = camera  # keep alive
            rd.camera = C.pointer(camera)
        return rd

    def render(self, sid: int, fid: int, rd: RenderDesc, wait: bool = True) -> RenderStats | None:
        self._ck(lib.rt_render(self._h, sid, fid, C.byref(rd)), "rt_render")
        return self.wait() if wait else None

    def wait(self) -> RenderStats:
        st = RenderStats()
        self._ck(lib.rt_render_wait(self._h, C.byref(st)), "rt_render_wait")
        return st

    def download(self, fid: int, w: int, h: int, planes: bool = True) -> dict:
        rgb = np.empty((h, w, 3), np.float32)
        rgb8 = np.empty((h, w, 3), np.uint8)
        obj = np.empty((h, w), np.int32) if planes else None
        prim = np.empty((h, w), np.int32) if planes else None
        t = np.empty((h, w), np.float32) if planes else None
        self._ck(lib.rt_frame_download(self._h, fid, _ptr(rgb), _ptr(rgb8), _ptr(obj), _ptr(prim), _ptr(t)),
                 "rt_frame_download")
        out = {"rgb": rgb, "rgb8": rgb8}
        if planes:
            out.update(obj=obj, prim=prim, t=t)
        return out

    def render_host(self, scene: SceneHost, rd: RenderDesc, w: int, h: int, want_rgb: bool = True,
                    rgb8: np.ndarray | None = None):
        rgb8 = np.empty((h, w, 3), np.uint8) if rgb8 is None else rgb8
        rgb = np.empty((h, w, 3), np.float32) if want_rgb else None
        st = RenderStats()
        self._ck(lib.rt_render_host(self._h, scene.desc_ptr(), C.byref(rd), _ptr(rgb8), _ptr(rgb), C.byref(st)),
                 "rt_render_host")
        return rgb, rgb8, st

    def batch(self, scenes, frames, rds, tuning: BatchTuning | None = None, plain: bool = False) -> None:
        n = len(scenes)
        s = np.asarray(scenes, np.int32)
        f = np.asarray(frames, np.int32)
        arr = (RenderDesc * n)(*rds)
        if plain:
            self._ck(lib.rt_batch_render_plain(self._h, n, _ptr(s), _ptr(f), C.cast(arr, P)), "rt_batch_render_plain")
        else:
            self._ck(lib.rt_batch_render(self._h, n, _ptr(s), _ptr(f), C.cast(arr, P),
                                         C.byref(tuning) if tuning is not None else None), "rt_batch_render")

    def autotune(self, scenes, frames, rds) -> BatchTuning:
        n = len(scenes)
        s = np.asarray(scenes, np.int32)
        f = np.asarray(frames, np.int32)
        arr = (RenderDesc * n)(*rds)
        t = BatchTuning()
        self._ck(lib.rt_batch_autotune(self._h, n, _ptr(s), _ptr(f), C.cast(arr, P), C.byref(t)), "rt_batch_autotune")
        return t

    def tuning(self) -> BatchTuning:
        """The plain path's current tuning."""
        t = BatchTuning()
        self._ck(lib.rt_ctx_get_tuning(self._h, C.byref(t)), "rt_ctx_get_tuning")
        return t

    def set_tuning(self, tuning: BatchTuning | None) -> None:
        self._ck(lib.rt_ctx_set_tuning(self._h, C.byref(tuning) if tuning is not None else None), "rt_ctx_set_tuning")

    def synchronize(self) -> None:
        self._ck(lib.rt_ctx_synchronize(self._h), "rt_ctx_synchronize")

    def release_cached(self) -> None:
        """Free the released scene and frame buffers the context keeps for reuse."""
        self._ck(lib.rt_ctx_release_cached(self._h), "rt_ctx_release_cached")

    def set_build(self, mode: int) -> None:
        """Hierarchy of the scenes built from now on: RT_BUILD_RADIX or RT_BUILD_CLUSTER."""
        self._ck(lib.rt_ctx_set_build(self._h, mode), "rt_ctx_set_build")

    def morton_sort(self, tri_p: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        tri_p = np.ascontiguousarray(tri_p, np.float32).reshape(-1, 9)
        n = tri_p.shape[0]
        codes = np.empty(n, np.uint32)
        perm = np.empty(n, np.uint32)
        self._ck(lib.rt_morton_sort(self._h, _ptr(tri_p), n, _ptr(codes), _ptr(perm)), "rt_morton_sort")
        return codes, perm

    def selftest_conversions(self, x: np.ndarray, d: float, v: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """The kernels' (float)((double)x * d) and llrint(v * 2^32), computed on the device."""
        x = np.ascontiguousarray(x, np.int64)
        v = np.ascontiguousarray(v, np.float32)
        assert x.shape == v.shape
        mul = np.empty(x.shape, np.float32)
        fix = np.empty(x.shape, np.int64)
        self._ck(lib.rt_selftest_conversions(self._h, _ptr(x), x.size, d, _ptr(v), _ptr(mul), _ptr(fix)),
                 "rt_selftest_conversions")
        return mul, fix

    def bvh(self, sid: int) -> tuple[np.ndarray, np.ndarray]:
        nn = C.c_int64()
        self._ck(lib.rt_scene_bvh_download(self._h, sid, None, None, C.byref(nn)), "rt_scene_bvh_download")
        nodes = np.empty((max(nn.value, 0), 8), np.float32)
        ntri = (nn.value + 1) // 2
        perm = np.empty(ntri, np.uint32)
        self._ck(lib.rt_scene_bvh_download(self._h, sid, _ptr(nodes), _ptr(perm), C.byref(nn)), "rt_scene_bvh_download")
        return nodes, perm

    def close(self) -> None:
        for ref in getattr(self, "_servers", []):   # servers live inside the context
            srv = ref()
            if srv is not None:
                srv.close()
        h, self._h = getattr(self, "_h", None), None
        if h:
            lib.rt_ctx_destroy(h)

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def orbit_camera(base: Camera, azimuth_deg: float, elevation_deg: float, width: int, height: int) -> Camera:
    """`base` moved about the world origin at its own distance, looking at the origin (rt_orbit_camera)."""
    out = Camera()
    rc = lib.rt_orbit_camera(C.byref(base), azimuth_deg, elevation_deg, width, height, C.byref(out))
    if rc:
        raise RTError(rc, "rt_orbit_camera")
    return out


class Server:
    """Continuous-batching render server over device-resident scenes (rt_server)."""

    def __init__(self, ctx: Context, budget_bytes: int, max_inflight: int = 64, max_level: int = 3, spp: int = 1,
                 plain: bool = False, queue_rays: int = 0, max_pixels: int = 0, keep_images: bool = True,
                 stages: int = 0):
        import weakref

        cfg = ServerConfig(int(budget_bytes), max_inflight, max_level, spp, int(plain), queue_rays, max_pixels,
                           int(keep_images), stages)
        h = P()
        rc = lib.rt_server_create(ctx.handle, C.byref(cfg), C.byref(h))
        if rc:
            raise RTError(rc, f"rt_server_create: {lib.rt_last_error(ctx.handle).decode(errors='replace')}")
        self._h, self._ctx, self.config = h, ctx, cfg
        self._cams: list[Camera] = []
        if not hasattr(ctx, "_servers"):
            ctx._servers = []
        ctx._servers.append(weakref.ref(self))

    def _ck(self, rc: int, what: str) -> None:
        if rc:
            raise RTError(rc, f"{what}: {lib.rt_server_last_error(self._h).decode(errors='replace')}")

    def set_tuning(self, tuning: BatchTuning | None) -> None:
        self._ck(lib.rt_server_set_tuning(self._h, C.byref(tuning) if tuning is not None else None),
                 "rt_server_set_tuning")

    def add_scene(self, scene: SceneHost) -> int:
        sid = C.c_int32()
        self._ck(lib.rt_server_add_scene(self._h, scene.desc_ptr(), C.byref(sid)), "rt_server_add_scene")
        cam = Camera()
        C.pointer(cam)[0] = scene.desc.camera
        self._cams.append(cam)
        return sid.value

    def camera(self, sid: int) -> Camera:
        return self._cams[sid]

    def submit(self, scene: int, width: int, height: int, camera: Camera | None = None, seed: int = 0,
               arrival_s: float = -1.0) -> int:
        if camera is None:   # the scene's own camera; an unknown scene is reported by the library
            camera = self._cams[scene] if 0 <= scene < len(self._cams) else Camera()
        req = Request(scene, width, height, camera, seed, arrival_s)
        rid = C.c_int64()
        self._ck(lib.rt_server_submit(self._h, C.byref(req), C.byref(rid)), "rt_server_submit")
        return rid.value

    def step(self) -> int:
        n = C.c_int32()
        self._ck(lib.rt_server_step(self._h, C.byref(n)), "rt_server_step")
        return n.value

    def drain(self) -> None:
        self._ck(lib.rt_server_drain(self._h), "rt_server_drain")

    def result(self, rid: int, image: bool = True) -> dict | None:
        """The finished request (with its image if kept), or None while it is queued or in flight."""
        res = RequestResult()
        rgb = rgb8 = None
        if image and self.config.keep_images:
            # the size is only known from the record: peek without images first is not possible
            # (taking the result forgets it), so allocate for the largest frame and trim
            n = int(self.config.max_pixels or 1920 * 1080)
            rgb, rgb8 = np.empty(3 * n, np.float32), np.empty(3 * n, np.uint8)
        rc = lib.rt_server_result(self._h, rid, C.byref(res), _ptr(rgb), _ptr(rgb8))
        if rc == RT_ERR_BUSY:
            return None
        self._ck(rc, "rt_server_result")
        out = res.as_dict()
        if rgb is not None and res.status == 0:
            npx = res.width * res.height
            out["rgb"] = rgb[: 3 * npx].reshape(res.height, res.width, 3)
            out["rgb8"] = rgb8[: 3 * npx].reshape(res.height, res.width, 3)
        return out

    def resident(self, sid: int) -> bool:
        r = C.c_int32()
        self._ck(lib.rt_server_resident(self._h, sid, C.byref(r)), "rt_server_resident")
        return bool(r.value)

    def now(self) -> float:
        return lib.rt_server_now(self._h)

    def stats(self) -> dict:
        st = ServeStats()
        self._ck(lib.rt_server_stats(self._h, C.byref(st)), "rt_server_stats")
        return st.as_dict()

    def latencies(self) -> np.ndarray:
        """Frame latencies (ms) behind the current stats."""
        n = C.c_int64()
        self._ck(lib.rt_server_latencies(self._h, None, 0, C.byref(n)), "rt_server_latencies")
        out = np.empty(n.value, np.float64)
        self._ck(lib.rt_server_latencies(self._h, _ptr(out), out.size, C.byref(n)), "rt_server_latencies")
        return out

    def wave_ms(self) -> np.ndarray:
        """Device time (ms) of each wave behind the current stats, in the order they ran."""
        n = C.c_int64()
        self._ck(lib.rt_server_wave_ms(self._h, None, 0, C.byref(n)), "rt_server_wave_ms")
        out = np.empty(n.value, np.float32)
        self._ck(lib.rt_server_wave_ms(self._h, _ptr(out), out.size, C.byref(n)), "rt_server_wave_ms")
        return out

    def run_poisson(self, lam: float, duration_s: float, seed: int = 4) -> dict:
        st = ServeStats()
        self._ck(lib.rt_server_run_poisson(self._h, lam, duration_s, seed, C.byref(st)), "rt_server_run_poisson")
        return st.as_dict()

    def close(self) -> None:
        h, self._h = getattr(self, "_h", None), None
        if h:
            lib.rt_server_destroy(h)

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
