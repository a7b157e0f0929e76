"""numpy mirrors of the C ABI structs in include/gbr.h.

The layouts are the reference's host/device structs byte for byte:
vertex 48 B (cl2.cl:131-138, vertex.hpp:33-63), triangle 144 B (cl2.cl:148-151),
obj_g_descriptor 144 B (cl2.cl:99-124, obj_g_descriptor.hpp), light 64 B
(cl2.cl:77-87, light.hpp).
"""
import numpy as np

VERTEX = np.dtype([
    ("pos", "<f4", 4), ("normal", "<f4", 4), ("vt", "<f4", 2),
    ("object_id", "<u4"), ("vertex_col", "<u4"),
])
TRIANGLE = np.dtype([("vertices", VERTEX, 3)])
OBJ_DESC = np.dtype([
    ("world_pos", "<f4", 4), ("world_rot_quat", "<f4", 4),
    ("old_world_pos_1", "<f4", 4), ("old_world_pos_2", "<f4", 4),
    ("old_world_rot_quat_1", "<f4", 4), ("old_world_rot_quat_2", "<f4", 4),
    ("scale", "<f4"), ("tid", "<u4"), ("rid", "<u4"), ("ssid", "<u4"),
    ("has_bump", "<u4"), ("specular", "<f4"), ("spec_mult", "<f4"), ("diffuse", "<f4"),
    ("buffer_offset", "<i4"), ("feature_flag", "<i4"), ("pad_", "<u4", 2),
])
LIGHT = np.dtype([
    ("pos", "<f4", 4), ("col", "<f4", 4), ("shadow", "<u4"), ("brightness", "<f4"),
    ("radius", "<f4"), ("diffuse", "<f4"), ("godray_intensity", "<f4"),
    ("is_static", "<i4"), ("pad_", "<u4", 2),
])
CAMERA = np.dtype([("pos", "<f4", 4), ("rot", "<f4", 4)])
# gbr_object_flush: what object::g_flush writes (48 bytes)
OBJECT_FLUSH = np.dtype([("index", "<u4"), ("tid", "<u4"), ("scale", "<f4"), ("feature_flag", "<i4"),
                         ("world_pos", "<f4", 4), ("world_rot_quat", "<f4", 4)])
VIEW = np.dtype([
    ("width", "<i4"), ("height", "<i4"), ("fov_const", "<f4"), ("hfov_deg", "<f4"),
    ("clear_col", "<f4", 4), ("use_linear", "<u4"), ("flags", "<u4"),
])
STATS = np.dtype([
    ("view_records", "<u8"), ("view_bin_entries", "<u8"), ("shadow_records", "<u8"),
    ("shadow_bin_entries", "<u8"), ("fragments_ref", "<u8"), ("retries", "<u8"),
    ("launches", "<u8"), ("stage_ms", "<f8", 10), ("stage_calls", "<u8", 10),
    ("view_samples", "<u8"), ("shadow_samples", "<u8"),
])
STAGES = ("shadow_setup", "shadow_scan", "shadow_fill", "shadow_raster",
          "view_setup", "view_scan", "view_fill", "view_raster", "view_shade")

SERVER_CONFIG = np.dtype([("hbm_budget_bytes", "<u8"), ("max_batch_views", "<u4"), ("max_batch_pixels", "<u4"),
                          ("max_inflight", "<u4"), ("batch_window_us", "<u4")])
REQUEST = np.dtype([
    ("scene", "<u4"), ("reserved", "<u4"), ("cam", CAMERA), ("view", VIEW),
    ("depth", "<u8"), ("id", "<u8"), ("rgba", "<u8"), ("user_tag", "<u8"),
])
COMPLETION = np.dtype([
    ("request_id", "<u8"), ("user_tag", "<u8"), ("status", "<i4"), ("batch_views", "<u4"),
    ("latency_ms", "<f8"), ("queue_ms", "<f8"),
])
SERVER_STATS = np.dtype([
    ("submitted", "<u8"), ("completed", "<u8"), ("rejected", "<u8"), ("batches", "<u8"),
    ("pixels_completed", "<u8"), ("peak_admitted_bytes", "<u8"), ("p50_ms", "<f8"), ("p99_ms", "<f8"),
    ("mean_ms", "<f8"), ("mean_batch_views", "<f8"), ("wall_s", "<f8"),
])

# gbr_tuning / gbr_batch_info (include/gbr.h)
TUNING = np.dtype([("raster_threads", "<i4"), ("coarse_tile", "<i4"), ("fine_max_tiles", "<i4"),
                   ("scratch_headroom", "<f4"), ("raster_shade", "<i4")])
RS_SEQUENTIAL, RS_FUSED, RS_PIPELINED = 0, 1, 2
BATCH_INFO = np.dtype([("views", "<u4"), ("graph_nodes", "<u4"), ("captures", "<u8"), ("launches", "<u8"),
                       ("reruns", "<u8"), ("scratch_bytes", "<u8")])
PASS_SHADOW, PASS_VIEW = 0, 1
BATCH_WITH_SHADOW = 1
DEFAULT_TUNING = {"raster_threads": 128, "coarse_tile": 128, "fine_max_tiles": 16, "scratch_headroom": 1.25,
                  "raster_shade": 0}


def make_tuning(raster_threads=128, coarse_tile=128, fine_max_tiles=16, scratch_headroom=1.25, raster_shade=0):
    t = np.zeros((), TUNING)
    t["raster_threads"] = raster_threads
    t["coarse_tile"] = coarse_tile
    t["fine_max_tiles"] = fine_max_tiles
    t["scratch_headroom"] = scratch_headroom
    t["raster_shade"] = raster_shade
    return t


assert VERTEX.itemsize == 48
assert TRIANGLE.itemsize == 144
assert OBJ_DESC.itemsize == 144
assert LIGHT.itemsize == 64
assert CAMERA.itemsize == 32
assert VIEW.itemsize == 40

# feature_flag bits (cl2.cl:90-97)
FLAG_TWO_SIDED = 2
FLAG_OUTLINE = 4
FLAG_IS_STATIC = 8
FLAG_NO_DYN_SHADOWS = 16


def make_descriptor(world_pos=(0, 0, 0), quat=(0, 0, 0, 1), scale=1.0, tid=0,
                    feature_flag=0, specular=0.9, spec_mult=1.0, diffuse=1.0):
    """One obj_g_descriptor with the reference's object defaults
    (object.cpp:72-74: specular 0.9, spec_mult 1, diffuse 1)."""
    d = np.zeros((), OBJ_DESC)
    d["world_pos"][:3] = world_pos
    d["world_rot_quat"][:] = quat
    d["old_world_pos_1"] = d["world_pos"]
    d["old_world_pos_2"] = d["world_pos"]
    d["old_world_rot_quat_1"] = d["world_rot_quat"]
    d["old_world_rot_quat_2"] = d["world_rot_quat"]
    d["scale"] = scale
    d["tid"] = tid
    d["rid"] = 0xFFFFFFFF
    d["ssid"] = 0xFFFFFFFF
    d["specular"] = specular
    d["spec_mult"] = spec_mult
    d["diffuse"] = diffuse
    d["feature_flag"] = feature_flag
    return d


def make_light(pos, col=(1, 1, 1), brightness=1.0, radius=20000.0, shadow=0, diffuse=1.0,
               is_static=0, godray_intensity=0.0):
    l = np.zeros((), LIGHT)
    l["pos"][:3] = pos
    l["col"][:3] = col
    l["shadow"] = shadow
    l["brightness"] = brightness
    l["radius"] = radius
    l["diffuse"] = diffuse
    l["is_static"] = is_static
    l["godray_intensity"] = godray_intensity
    return l


def make_camera(pos=(0, 0, 0), rot=(0, 0, 0)):
    c = np.zeros((), CAMERA)
    c["pos"][:3] = pos
    c["rot"][:3] = rot
    return c


VIEW_NORMAL_MAPPING = 1
VIEW_OUTLINE = 2


def make_view(width, height, hfov_deg=90.0, fov_const=0.0, clear=(0, 0, 0, 1), use_linear=1, flags=0):
    v = np.zeros((), VIEW)
    v["flags"] = flags
    v["width"] = width
    v["height"] = height
    v["hfov_deg"] = hfov_deg
    v["fov_const"] = fov_const
    v["clear_col"][:] = clear
    v["use_linear"] = use_linear
    return v
