"""ctypes mirror of include/salvia_gb300.h.

The structures below are field-for-field copies of the C descriptors; the
`bind()` helper attaches argtypes/restype to every entry point of a loaded
library that exports the ABI.
"""
import ctypes as C

SG_OK, SG_FAILED, SG_OUT_OF_MEMORY, SG_INVALID_PARAMETER, SG_TIMEOUT, SG_CUDA_ERROR = range(6)
STATUS_NAMES = {0: "ok", 1: "failed", 2: "out_of_memory", 3: "invalid_parameter",
                4: "timeout", 5: "cuda_error"}

SG_MAX_VS_INPUTS = 8
SG_MAX_VARYINGS = 5
SG_MAX_STREAMS = 8
SG_MAX_SHADER_CONSTANTS = 48
SG_MAX_SHADER_SAMPLERS = 2

TOPOLOGY_LINE_LIST, TOPOLOGY_LINE_STRIP, TOPOLOGY_TRIANGLE_LIST, TOPOLOGY_TRIANGLE_STRIP = 0, 1, 2, 4
CULL_NONE, CULL_FRONT, CULL_BACK = 0, 1, 2
FILL_WIREFRAME, FILL_SOLID = 0, 1
CMP_NEVER, CMP_LESS, CMP_EQUAL, CMP_LESS_EQUAL, CMP_GREATER, CMP_NOT_EQUAL, \
    CMP_GREATER_EQUAL, CMP_ALWAYS = range(8)
SOP_KEEP, SOP_ZERO, SOP_REPLACE, SOP_INCR_SAT, SOP_DECR_SAT, SOP_INVERT, SOP_INCR_WRAP, \
    SOP_DECR_WRAP = range(1, 9)
FILTER_POINT, FILTER_LINEAR, FILTER_ANISOTROPIC = 0, 1, 2
ADDRESS_WRAP, ADDRESS_MIRROR, ADDRESS_CLAMP, ADDRESS_BORDER = 0, 1, 2, 3
MIP_LO_QUALITY, MIP_MI_QUALITY, MIP_HI_QUALITY = 0, 1, 2
CLEAR_DEPTH, CLEAR_STENCIL = 1, 2
FMT_RGBA32F, FMT_RGB32F, FMT_BGRA8, FMT_RGBA8, FMT_R32F, FMT_RG32F, FMT_R32I = range(7)
FMT_RGBA16F, FMT_D32F, FMT_D24S8 = 16, 17, 18
FORMAT_BYTES = {FMT_RGBA32F: 16, FMT_RGB32F: 12, FMT_BGRA8: 4, FMT_RGBA8: 4, FMT_R32F: 4,
                FMT_RG32F: 8, FMT_R32I: 4, FMT_RGBA16F: 8, FMT_D32F: 4, FMT_D24S8: 4}
VFMT_R32G32B32A32_FLOAT, VFMT_R32G32B32A32_SINT, VFMT_R32G32B32_FLOAT = 2, 4, 6
VFMT_R32G32_FLOAT, VFMT_R32_FLOAT = 16, 41
INDEX_U32, INDEX_U16 = 42, 57
AM_LINEAR, AM_CENTROID, AM_NOINTERPOLATION, AM_NOPERSPECTIVE, AM_SAMPLE = 1, 2, 4, 8, 16
SEMANTIC_POSITION, SEMANTIC_TEXCOORD, SEMANTIC_COLOR, SEMANTIC_NORMAL = 0, 1, 2, 3

VS_TRANSFORM, VS_MORPH_DISPLACE = 1, 2
PS_COLOR, PS_CONSTANT, PS_TEX_MODULATE, PS_TEX_GRAD_MODULATE, PS_TEX_GRAD_LEARNED = 1, 2, 3, 4, 5
PS_TEX_LOD_MODULATE, PS_TEX_PROJ_MODULATE, PS_TEX_ALPHA_TEST, PS_COLOR_MRT, PS_TEXCUBE_MODULATE = 6, 7, 8, 9, 10
TEXTURED_PS = (PS_TEX_MODULATE, PS_TEX_GRAD_MODULATE, PS_TEX_GRAD_LEARNED, PS_TEX_LOD_MODULATE, PS_TEX_PROJ_MODULATE,
               PS_TEX_ALPHA_TEST, PS_TEXCUBE_MODULATE)
BS_REPLACE, BS_LERP_SRC_ALPHA, BS_ADD, BS_REPLACE_ALL = 1, 2, 3, 4
MAX_COLOR_TARGETS = 7
CMD_DRAW, CMD_CLEAR_COLOR, CMD_CLEAR_DEPTH_STENCIL, CMD_RESOLVE = 1, 2, 3, 4


class Viewport(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("w", C.c_float), ("h", C.c_float),
                ("minz", C.c_float), ("maxz", C.c_float)]


class RasterDesc(C.Structure):
    _fields_ = [("fill_mode", C.c_uint32), ("cull_mode", C.c_uint32),
                ("front_ccw", C.c_uint32), ("reserved", C.c_uint32)]


class StencilFaceDesc(C.Structure):
    _fields_ = [("fail_op", C.c_uint32), ("depth_fail_op", C.c_uint32),
                ("pass_op", C.c_uint32), ("func", C.c_uint32)]


class DepthStencilDesc(C.Structure):
    _fields_ = [("depth_enable", C.c_uint32), ("depth_write", C.c_uint32),
                ("depth_func", C.c_uint32), ("stencil_enable", C.c_uint32),
                ("stencil_read_mask", C.c_uint32), ("stencil_write_mask", C.c_uint32),
                ("front", StencilFaceDesc), ("back", StencilFaceDesc)]


class SamplerDesc(C.Structure):
    _fields_ = [("min_filter", C.c_uint32), ("mag_filter", C.c_uint32),
                ("mip_filter", C.c_uint32), ("mip_quality", C.c_uint32),
                ("address_u", C.c_uint32), ("address_v", C.c_uint32),
                ("address_w", C.c_uint32), ("max_anisotropy", C.c_uint32),
                ("lod_bias", C.c_float), ("border_color", C.c_float * 4),
                ("min_lod", C.c_float), ("max_lod", C.c_float)]


class VertexStream(C.Structure):
    _fields_ = [("buffer", C.c_uint32), ("stride", C.c_uint32), ("offset", C.c_uint32)]


class VSInput(C.Structure):
    _fields_ = [("semantic", C.c_uint32), ("semantic_index", C.c_uint32),
                ("format", C.c_uint32), ("slot", C.c_uint32), ("offset", C.c_uint32)]


class Shader(C.Structure):
    _fields_ = [("program", C.c_uint32), ("samplers", C.c_uint32 * SG_MAX_SHADER_SAMPLERS),
                ("learned_filter", C.c_uint32), ("constants", C.c_float * SG_MAX_SHADER_CONSTANTS)]


class DrawDesc(C.Structure):
    _fields_ = [("color_target", C.c_uint32), ("ds_target", C.c_uint32),
                ("viewport", Viewport), ("topology", C.c_uint32), ("indexed", C.c_uint32),
                ("index_buffer", C.c_uint32), ("index_format", C.c_uint32),
                ("start", C.c_uint32), ("prim_count", C.c_uint32), ("base_vertex", C.c_int32),
                ("num_streams", C.c_uint32), ("streams", VertexStream * SG_MAX_STREAMS),
                ("num_inputs", C.c_uint32), ("inputs", VSInput * SG_MAX_VS_INPUTS),
                ("num_varyings", C.c_uint32),
                ("varying_modifiers", C.c_uint32 * SG_MAX_VARYINGS),
                ("raster", RasterDesc), ("depth_stencil", DepthStencilDesc),
                ("stencil_ref", C.c_int32), ("vs", Shader), ("ps", Shader), ("bs", Shader),
                ("more_color_targets", C.c_uint32 * 6)]


class ProfileData(C.Structure):
    _fields_ = [("geometry_ms", C.c_double), ("binning_ms", C.c_double), ("raster_ms", C.c_double),
                ("cover_ms", C.c_double), ("shade_ms", C.c_double), ("merge_ms", C.c_double),
                ("draws", C.c_uint64), ("launches", C.c_uint64), ("raster_launches", C.c_uint64),
                ("af_lookups", C.c_uint64), ("af_fallbacks", C.c_uint64), ("cover_batches", C.c_uint64),
                ("cover_rounds", C.c_uint64), ("cover_pairs", C.c_uint64)]


class DrawStats(C.Structure):
    _fields_ = [("ia_primitives", C.c_uint64), ("cprimitives", C.c_uint64),
                ("ps_invocations", C.c_uint64), ("backend_input_pixels", C.c_uint64),
                ("ia_vertices", C.c_uint64), ("vs_invocations", C.c_uint64), ("cinvocations", C.c_uint64)]


# counters whose values the reference renderer fixes (vs_invocations depends
# on its worker threads' vertex caches)
REFERENCE_STATS = ("ia_primitives", "cprimitives", "ps_invocations", "backend_input_pixels", "ia_vertices",
                   "cinvocations")


class Command(C.Structure):
    _fields_ = [("type", C.c_uint32), ("texture", C.c_uint32), ("texture2", C.c_uint32),
                ("flags", C.c_uint32), ("color", C.c_float * 4), ("depth", C.c_float),
                ("stencil", C.c_uint32), ("draw", C.POINTER(DrawDesc))]


class Tuning(C.Structure):
    _fields_ = [("cover_item", C.c_uint32), ("split_entries", C.c_uint32), ("bin_chunk", C.c_uint32),
                ("bin_capacity", C.c_uint32), ("frag_chunks", C.c_uint32),
                ("shade_quads_per_warp", C.c_uint32), ("shade_ctas_per_sm", C.c_uint32),
                ("merge_ctas_per_sm", C.c_uint32), ("cover_threads_per_block", C.c_uint32),
                ("cover_ctas_per_sm", C.c_uint32), ("shade_resident", C.c_uint32),
                ("merge_resident", C.c_uint32)]


class TuningKnob(C.Structure):
    """sg_tuning_knob"""
    _fields_ = [("field", C.c_char_p), ("count", C.c_uint32), ("values", C.c_uint32 * 8)]


_u32p = C.POINTER(C.c_uint32)

class AfTrainDesc(C.Structure):
    """sg_af_train_desc"""
    _fields_ = [("samplers", _u32p), ("num_samplers", C.c_uint32), ("samples", C.c_uint32),
                ("batch", C.c_uint32), ("epochs", C.c_uint32), ("lr", C.c_float), ("seed", C.c_uint64)]


class AfReport(C.Structure):
    """sg_af_report"""
    _fields_ = [("first_loss", C.c_float), ("last_loss", C.c_float), ("steps", C.c_uint32),
                ("train_ms", C.c_float)]


class Image(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("channels", C.c_uint32),
                ("reserved", C.c_uint32), ("pixels", C.POINTER(C.c_uint8))]


class Blob(C.Structure):
    _fields_ = [("data", C.POINTER(C.c_uint8)), ("size", C.c_size_t)]


class ObjMaterial(C.Structure):
    _fields_ = [("name", C.c_char_p), ("tex_name", C.c_char_p), ("tex_path", C.c_char_p),
                ("ambient", C.c_float * 4), ("diffuse", C.c_float * 4), ("specular", C.c_float * 4),
                ("shininess", C.c_int32), ("alpha", C.c_float), ("is_specular", C.c_int32),
                ("first_index", C.c_uint32), ("index_count", C.c_uint32), ("reserved", C.c_uint32)]


class ObjMesh(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("num_indices", C.c_uint32), ("num_materials", C.c_uint32),
                ("reserved", C.c_uint32), ("vertices", C.POINTER(C.c_float)), ("indices", C.POINTER(C.c_uint32)),
                ("materials", C.POINTER(ObjMaterial))]


SIGNATURES = {
    "sg_device_create": (C.c_int32, [C.c_int32, C.c_void_p, C.POINTER(C.c_void_p)]),
    "sg_device_destroy": (None, [C.c_void_p]),
    "sg_sync": (C.c_int32, [C.c_void_p]),
    "sg_last_error": (C.c_char_p, [C.c_void_p]),
    "sg_profile_enable": (C.c_int32, [C.c_void_p, C.c_int32]),
    "sg_profile_read": (C.c_int32, [C.c_void_p, C.POINTER(ProfileData)]),
    "sg_buffer_create": (C.c_int32, [C.c_void_p, C.c_size_t, _u32p]),
    "sg_buffer_upload": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_size_t, C.c_void_p, C.c_size_t]),
    "sg_buffer_download": (C.c_int32,
                           [C.c_void_p, C.c_uint32, C.c_size_t, C.c_void_p, C.c_size_t]),
    "sg_buffer_destroy": (C.c_int32, [C.c_void_p, C.c_uint32]),
    "sg_texture_create": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                      C.c_uint32, _u32p]),
    "sg_texture_upload": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                      C.c_size_t]),
    "sg_texture_download": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                        C.c_size_t]),
    "sg_texture_gen_mipmap": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "sg_texture_info": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32, _u32p, _u32p, _u32p,
                                    _u32p, _u32p]),
    "sg_texture_destroy": (C.c_int32, [C.c_void_p, C.c_uint32]),
    "sg_sampler_create": (C.c_int32, [C.c_void_p, C.POINTER(SamplerDesc), C.c_uint32, _u32p]),
    "sg_sampler_destroy": (C.c_int32, [C.c_void_p, C.c_uint32]),
    "sg_draw": (C.c_int32, [C.c_void_p, C.POINTER(DrawDesc), C.POINTER(DrawStats)]),
    "sg_shader_register": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint32)]),
    "sg_texture_create_cube": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                           C.POINTER(C.c_uint32)]),
    "sg_draw_static_scratch": (C.c_int32, [C.c_void_p, C.POINTER(DrawDesc), C.POINTER(DrawStats)]),
    "sg_clear_color": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(C.c_float)]),
    "sg_clear_depth_stencil": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_float,
                                           C.c_uint32]),
    "sg_resolve": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "sg_submit": (C.c_int32, [C.c_void_p, C.POINTER(Command), C.c_uint32, C.POINTER(DrawStats)]),
    "sg_graph_create": (C.c_int32, [C.c_void_p, C.POINTER(Command), C.c_uint32, C.POINTER(C.c_void_p)]),
    "sg_graph_launch": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "sg_graph_info": (C.c_int32, [C.c_void_p, C.c_void_p, _u32p, _u32p]),
    "sg_graph_destroy": (None, [C.c_void_p, C.c_void_p]),
    "sg_get_tuning": (C.c_int32, [C.c_void_p, C.POINTER(Tuning)]),
    "sg_set_tuning": (C.c_int32, [C.c_void_p, C.POINTER(Tuning)]),
    "sg_autotune": (C.c_int32, [C.c_void_p, C.POINTER(Command), C.c_uint32, C.c_uint32,
                                C.POINTER(Tuning), C.POINTER(C.c_float)]),
    "sg_autotune_space": (C.c_int32, [C.POINTER(C.POINTER(TuningKnob)), C.POINTER(C.c_uint32)]),
    "sg_af_model_create": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "sg_af_model_destroy": (None, [C.c_void_p, C.c_void_p]),
    "sg_af_model_id": (C.c_uint32, [C.c_void_p]),
    "sg_af_model_get_params": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(C.c_float)]),
    "sg_af_model_set_params": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(C.c_float)]),
    "sg_af_model_forward": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(C.c_float), C.c_uint32,
                                        C.POINTER(C.c_float)]),
    "sg_af_sample": (C.c_int32, [C.c_void_p, _u32p, C.c_uint32, C.c_uint32, C.c_uint64,
                                 C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "sg_af_model_gradients": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                          C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "sg_af_make_textures": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, _u32p]),
    "sg_af_model_train": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(AfTrainDesc), C.POINTER(AfReport)]),
    "sg_image_decode": (C.c_int32, [C.c_void_p, C.c_size_t, C.POINTER(Image)]),
    "sg_image_release": (None, [C.POINTER(Image)]),
    "sg_blob_release": (None, [C.POINTER(Blob)]),
    "sg_image_encode_png": (C.c_int32, [C.POINTER(Image), C.POINTER(Blob)]),
    "sg_image_encode_hdr": (C.c_int32, [C.POINTER(C.c_float), C.c_uint32, C.c_uint32, C.POINTER(Blob)]),
    "sg_texture_write_image": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(Image)]),
    "sg_texture_encode_image": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(Blob)]),
    "sg_obj_load": (C.c_int32, [C.c_char_p, C.c_int32, C.POINTER(C.POINTER(ObjMesh))]),
    "sg_obj_release": (None, [C.POINTER(ObjMesh)]),
    "sg_sasl_translate": (C.c_int32, [C.c_char_p, C.c_uint32, C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p),
                                      C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "sg_sasl_free": (None, [C.c_void_p]),
}

AF_FEATURES, AF_OUTPUTS, AF_PARAMS = 24, 5, 6085

# Entry points of the GPU library with no counterpart in the reference (the
# CPU oracle does not export them).
PRODUCT_ONLY = {"sg_draw_static_scratch", "sg_graph_create", "sg_graph_launch", "sg_graph_info",
                "sg_graph_destroy", "sg_get_tuning", "sg_set_tuning", "sg_autotune", "sg_autotune_space"}
PRODUCT_ONLY |= {name for name in SIGNATURES if name.startswith("sg_af_")}

# Image and mesh ingest (tex_io.cpp, mesh_io_obj.cpp): host codecs and the
# OBJ loader in the GPU library; the draw oracle does not export them (their
# checkers are oracle/ingest_oracle.py and the reference's own loader).
INGEST = {"sg_image_decode", "sg_image_release", "sg_blob_release", "sg_image_encode_png", "sg_image_encode_hdr",
          "sg_texture_write_image", "sg_texture_encode_image", "sg_obj_load", "sg_obj_release"}

# The SASL translator (renderer.h compile()): host code of the GPU library;
# the draw oracle runs the modules it makes, built for the host.
SASL = {"sg_sasl_translate", "sg_sasl_free"}
LANG_VERTEX_SHADER = 2
LANG_PIXEL_SHADER = 3


def bind(lib, extra=None):
    """Attach the ABI's signatures to the functions exported by `lib`."""
    sigs = dict(SIGNATURES)
    if extra:
        sigs.update(extra)
    for name, (restype, argtypes) in sigs.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = restype
        fn.argtypes = argtypes
    return lib
