/*
 * salvia_gb300.h -- C ABI of the GB300 rasterization pipeline.
 *
 * This is the drop-in boundary for Salvia's draw path.  Every entry point
 * below replaces one call of the reference C++ renderer interface
 * (salvia/include/salvia/core/renderer.h:42-147) with a plain-pointer,
 * plain-size C function; the C++ facade in salvia_gb300/renderer.hpp maps the
 * reference's classes (renderer, raster_state, depth_stencil_state, sampler,
 * input_layout, cpp_*_shader) onto it.
 *
 * Conventions
 *  - Status codes mirror `enum class result` (salvia/include/salvia/common/
 *    constants.h:9): SG_OK, SG_FAILED, SG_OUT_OF_MEMORY, SG_INVALID_PARAMETER,
 *    plus SG_TIMEOUT for bounded device waits and SG_CUDA_ERROR.
 *  - Enumerations keep the reference's numeric values (primitive topology,
 *    cull mode, compare function, stencil op, filter, address mode, pixel
 *    format, index format) so a caller can pass the reference's enums through.
 *  - Resources are addressed by 32-bit handles; handle 0 means "none".
 *  - All calls are stream-ordered on the device's CUDA stream; only the
 *    *_download / sg_sync calls block the host.
 *  - No call takes or returns a torch or CUDA type: streams are `void*`.
 */
#ifndef SALVIA_GB300_H
#define SALVIA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status ------------------------------------------------------------- */
enum {
  SG_OK = 0,
  SG_FAILED = 1,
  SG_OUT_OF_MEMORY = 2,
  SG_INVALID_PARAMETER = 3,
  SG_TIMEOUT = 4,
  SG_CUDA_ERROR = 5
};

/* ---- capacities (salvia/include/salvia/common/renderer_capacity.h) ------- */
#define SG_MAX_VS_INPUTS 8    /* MAX_VS_INPUT_ATTRS */
#define SG_MAX_VARYINGS 5     /* vs_output op table covers 0..5 attributes (shader.cpp:45-78) */
#define SG_MAX_STREAMS 8
#define SG_MAX_RT_SIZE 8192   /* MAX_RENDER_TARGET_WIDTH/HEIGHT */
#define SG_MAX_SHADER_CONSTANTS 48
#define SG_MAX_SHADER_SAMPLERS 2
/* colour targets of one draw: set_render_targets takes fewer than
 * MAX_RENDER_TARGETS = 8 (renderer_impl.cpp:159-238) */
#define SG_MAX_COLOR_TARGETS 7

/* ---- enumerations (reference numeric values) ----------------------------- */
/* primitive_topology (constants.h:44-52) */
enum {
  SG_TOPOLOGY_LINE_LIST = 0, SG_TOPOLOGY_LINE_STRIP = 1,
  SG_TOPOLOGY_TRIANGLE_LIST = 2, SG_TOPOLOGY_TRIANGLE_STRIP = 4
};
/* cull_mode (constants.h:58-63) */
enum { SG_CULL_NONE = 0, SG_CULL_FRONT = 1, SG_CULL_BACK = 2 };
/* fill_mode (constants.h:66-70) */
enum { SG_FILL_WIREFRAME = 0, SG_FILL_SOLID = 1 };

/* Lines and wireframe.  The reference declares line topologies and
 * fill_wireframe but stops at ef_unimplemented (rasterizer.cpp:1019-1060,
 * clipper.cpp:39-41); its rasterize_line (rasterizer.cpp:60-213) holds the
 * intended DDA.  This library defines them as follows.
 *   - Assembly: a line list takes vertices (2p, 2p + 1) for primitive p, a
 *     strip (p, p + 1), through the index buffer as triangles do.  A
 *     triangle topology with SG_FILL_WIREFRAME is assembled, clipped and
 *     culled as a solid triangle; each triangle it yields is drawn as its
 *     three edges (a, b), (b, c), (c, a).
 *   - Clipping: a segment is cut at z >= 0, then at z <= w, the outside end
 *     replaced by lerp(inside, outside, d_in / (d_in - d_out)), as the
 *     triangle clipper does; lines are not culled.
 *   - Rasterization: rasterize_line's DDA over the draw's viewport within
 *     the render area, every pixel once: along the major axis (x when
 *     |dx| > |dy|), from the end with the smaller coordinate, the pixels
 *     i in [fast_floori(fast_floor(start + 0.5)), fast_floori(end - 0.5)),
 *     both ends clamped to the viewport's [lo, hi] (rasterize_line clamps
 *     the start to hi - 1, which would add an extrapolated pixel to a line
 *     starting past the far edge); pixel i takes the endpoints' registers
 *     lerped at t = (i + 0.5 - start) / (end - start), its minor
 *     coordinate floori(t-lerped minor) (pixels outside the viewport are
 *     skipped), depth the lerped z, attributes unprojected by the lerped w.
 *   - Pixel shading: once per pixel; ddx / ddy of an attribute are its
 *     values at the lerped registers plus the line's ddx / ddy (rasterize_
 *     line's diff * (diff.x / |diff.xy|^2), diff * (diff.y / |diff.xy|^2))
 *     minus its value at the pixel.  User pixel and blend shaders are not
 *     taken (SG_INVALID_PARAMETER); learned-filter draws sample plainly.
 *   - Output: sample 0 of the pixel (render_sample(..., 0, ...)), with the
 *     depth and stencil tests after shading and the front-face stencil
 *     state.  Pipeline counters: cprimitives counts the segments drawn,
 *     ps_invocations and backend_input_pixels the pixels shaded. */
/* compare_function (constants.h:143-152) */
enum {
  SG_CMP_NEVER = 0, SG_CMP_LESS = 1, SG_CMP_EQUAL = 2, SG_CMP_LESS_EQUAL = 3,
  SG_CMP_GREATER = 4, SG_CMP_NOT_EQUAL = 5, SG_CMP_GREATER_EQUAL = 6, SG_CMP_ALWAYS = 7
};
/* stencil_op (constants.h:154-163) */
enum {
  SG_SOP_KEEP = 1, SG_SOP_ZERO = 2, SG_SOP_REPLACE = 3, SG_SOP_INCR_SAT = 4,
  SG_SOP_DECR_SAT = 5, SG_SOP_INVERT = 6, SG_SOP_INCR_WRAP = 7, SG_SOP_DECR_WRAP = 8
};
/* filter_type / address_mode / mip_quality (constants.h:82-102) */
enum { SG_FILTER_POINT = 0, SG_FILTER_LINEAR = 1, SG_FILTER_ANISOTROPIC = 2 };
enum { SG_ADDRESS_WRAP = 0, SG_ADDRESS_MIRROR = 1, SG_ADDRESS_CLAMP = 2, SG_ADDRESS_BORDER = 3 };
enum { SG_MIP_LO_QUALITY = 0, SG_MIP_MI_QUALITY = 1, SG_MIP_HI_QUALITY = 2 };
/* clear_flag (constants.h:165) */
enum { SG_CLEAR_DEPTH = 1, SG_CLEAR_STENCIL = 2 };
/* pixel formats: the reference's pixel_format codes (colors_convertors.h:39-45)
 * plus three formats the reference does not have (documented extensions). */
enum {
  SG_FMT_RGBA32F = 0, SG_FMT_RGB32F = 1, SG_FMT_BGRA8 = 2, SG_FMT_RGBA8 = 3,
  SG_FMT_R32F = 4, SG_FMT_RG32F = 5, SG_FMT_R32I = 6,
  SG_FMT_RGBA16F = 16,   /* extension: half colour, round-to-nearest-even */
  SG_FMT_D32F = 17,      /* extension: float depth, no stencil */
  SG_FMT_D24S8 = 18      /* extension: 24-bit unorm depth (low) + 8-bit stencil (high) */
};
/* vertex element formats (salvia/include/salvia/common/format.h) */
enum {
  SG_VFMT_R32G32B32A32_FLOAT = 2, SG_VFMT_R32G32B32A32_SINT = 4, SG_VFMT_R32G32B32_FLOAT = 6,
  SG_VFMT_R32G32_FLOAT = 16, SG_VFMT_R32_FLOAT = 41
};
/* index formats */
enum { SG_INDEX_U32 = 42, SG_INDEX_U16 = 57 };
/* vs_output::attrib_modifier_type (shader_regs.h:49-55) */
enum {
  SG_AM_LINEAR = 1, SG_AM_CENTROID = 2, SG_AM_NOINTERPOLATION = 4,
  SG_AM_NOPERSPECTIVE = 8, SG_AM_SAMPLE = 16
};
/* semantic of a vertex-shader input register: POSITION fills w with 1 when
 * the element has fewer than four components, anything else with 0
 * (salvia/include/salvia/shader/constants.h:119). */
enum { SG_SEMANTIC_POSITION = 0, SG_SEMANTIC_TEXCOORD = 1, SG_SEMANTIC_COLOR = 2, SG_SEMANTIC_NORMAL = 3 };

/* ---- stock shader programs --------------------------------------------------
 * The reference runs user C++ virtual shaders on the CPU (shader.h:159-215).
 * Device code cannot call host virtuals, so the ABI names compiled device
 * programs; their bodies are written once per program and documented here
 * with the reference call each one makes.                                   */
enum {
  /* out.position = transform(in[0], M)  (eflib::transform row-vector x matrix,
   * eflib/src/math.cpp:142-154); out.attr[i] = in[i+1] for i < num_varyings.
   * constants[0..15] = M, row-major (m[r][c] at 4r+c). */
  SG_VS_TRANSFORM = 1,
  /* Morph + vertex-texture displacement (the VertexTextureFetch/Morph
   * samples' pattern): p = p0 + (p1 - p0) * k[16]; n = in[2];
   * h = vs_sampler0.sample(in[3].x, in[3].y, 0).r; p.xyz += n.xyz * (h * k[17]);
   * out.position = transform(p, M); out.attr[0] = in[3]; out.attr[1] = n;
   * constants[0..15] = M, k[16] = morph weight, k[17] = displacement scale. */
  SG_VS_MORPH_DISPLACE = 2
};
enum {
  SG_PS_COLOR = 1,          /* out.color[0] = in.attr[0] */
  SG_PS_CONSTANT = 2,       /* out.color[0] = constants[0..3] */
  /* out.color[0] = tex2d(sampler0, 0) * in.attr[1]; tex2d computes the LOD
   * once per quad from quad differences (cpp_pixel_shader.cpp:23-31). */
  SG_PS_TEX_MODULATE = 3,
  /* out.color[0] = sampler0.sample_2d_grad(in.attr[0].xy, ddx(0).xy,
   * ddy(0).xy, 0) * in.attr[1]  (sampler.cpp:854-873; the anisotropic path). */
  SG_PS_TEX_GRAD_MODULATE = 4,
  /* No counterpart in the reference: SG_PS_TEX_GRAD_MODULATE with the
   * anisotropic lookup approximated by the learned filter named in the
   * shader's `learned_filter` (sg_af_model_id) where it applies -- a minified
   * lookup of an anisotropic sampler with more than constants[2] and at most
   * constants[1] probes -- and where the filter's confidence is at least
   * constants[0]; every other lookup runs the plain sampler. */
  SG_PS_TEX_GRAD_LEARNED = 5,
  /* out.color[0] = tex2dlod(sampler0, 0) * in.attr[1]: the lookup at
   * (attr[0].x, attr[0].y) with attr[0].w as the mip level, sampler::sample
   * (cpp_pixel_shader.cpp:33-40). */
  SG_PS_TEX_LOD_MODULATE = 6,
  /* out.color[0] = tex2dproj(sampler0, 0) * in.attr[1]: attr[0] divided by
   * its w and mapped from [-1, 1] to [0, 1], with the derivatives of that
   * projection across the quad (cpp_pixel_shader.cpp:42-60). */
  SG_PS_TEX_PROJ_MODULATE = 7,
  /* out.color[0] = c = tex2d(sampler0, 0) * in.attr[1]; discard
   * (shader_prog returns false) when c.a < constants[0] -- the alpha-test
   * pattern.  As in the reference, a quad keeps pixel 0 when pixel 0 or
   * pixel 2 passes and pixels 1-3 when pixel 1 or pixel 3 passes (the pass
   * mask is built from int shifts, cpp_pixel_shader.cpp:62-74); a pixel that
   * is not kept is neither blended nor depth-tested late, and with early-Z
   * its depth was already written (rasterizer.cpp:1245-1421). */
  SG_PS_TEX_ALPHA_TEST = 8,
  /* out.color[i] = in.attr[i] for every varying i (one colour per bound
   * target); colours a program does not write are zero. */
  SG_PS_COLOR_MRT = 9,
  /* out.color[0] = sampler0.sample_cube(attr[0].x, attr[0].y, attr[0].z,
   * attr[0].w) * in.attr[1]: the direction's major axis picks the face
   * (sampler.cpp:771-829).  The reference declares the texcube helpers
   * (shader.h:187-198) but defines none, so the program calls the sampler. */
  SG_PS_TEXCUBE_MODULATE = 10
};
enum {
  SG_BS_REPLACE = 1,        /* color(0, s) = in.color[0] */
  SG_BS_LERP_SRC_ALPHA = 2, /* color(0, s) = lerp(dst, src, src.a) (TextureAndBlending.cpp:168-176) */
  SG_BS_ADD = 3,            /* color(0, s) = dst + src */
  SG_BS_REPLACE_ALL = 4     /* color(i, s) = in.color[i] for every bound colour target i */
};

/* ---- user shader programs ----------------------------------------------------
 * The reference's applications write shader bodies as C++ classes
 * (cpp_vertex_shader / cpp_pixel_shader / cpp_blend_shader, shader.h:159-215).
 * Here a shader body is a class compiled by the application with nvcc
 * against <salvia_gb300/device_shader.cuh> and exported by
 * SALVIA_GB300_VERTEX_SHADER, SALVIA_GB300_PIXEL_SHADER or
 * SALVIA_GB300_BLEND_SHADER as an sg_shader_module: the pass kernels
 * instantiated for the class (device code in the application's own module),
 * and the same body compiled for the host, which CPU backends of this ABI
 * run.  sg_shader_register gives the module a program id (at least
 * SG_USER_PROGRAM_BASE) that draws name in sg_shader.program, beside the
 * stock SG_VS_* / SG_PS_* / SG_BS_* programs.  Vertex shaders read sampler
 * slot 0 and the constants of the draw's vertex shader; pixel shaders those
 * of its pixel shader; blend shaders the blend shader's constants.  A pass
 * holds draws of at most one user vertex shader, 8 user pixel shaders and
 * one user blend shader (more split the pass). */
#define SG_SHADER_ABI_VERSION 2
#define SG_USER_PROGRAM_BASE 64
enum { SG_STAGE_PIXEL = 1, SG_STAGE_BLEND = 2, SG_STAGE_VERTEX = 3 };

/* What a host backend hands a vertex-shader body for one vertex
 * (cpp_vertex_shader::execute, shader.cpp:520-522): the fetched input
 * registers (vs_input, stream_assembler.cpp:26-93) and the backend's
 * sampler::sample for vertex texture fetch (sampler slot 0 of the draw's
 * vertex shader); the body writes the position and the varyings. */
typedef struct sg_host_vs_io {
  float in[SG_MAX_VS_INPUTS][4];       /* vs_input::attribute(i) */
  uint32_t num_varyings;
  const float* constants;              /* the vertex shader's SG_MAX_SHADER_CONSTANTS */
  void* backend;
  void (*sample)(void* backend, float u, float v, float lod, float out[4]);  /* sampler::sample */
  float position[4];                   /* out: vs_output::position() */
  float attr[SG_MAX_VARYINGS][4];      /* out: vs_output::attribute(i) */
} sg_host_vs_io;

/* What a host backend hands a pixel-shader body for one pixel of a quad
 * (cpp_pixel_shader::execute, cpp_pixel_shader.cpp:62-74): the pixel's
 * interpolated registers and the backend's own cpp_pixel_shader helpers
 * (cpp_pixel_shader.cpp:13-60; `reg` is a varying index, the lookups use
 * sampler slot 0 of the draw's pixel shader). */
typedef struct sg_host_ps_io {
  float attr[SG_MAX_VARYINGS][4];      /* vs_output::attribute(i) */
  float position[4];
  uint32_t front_face;
  uint32_t num_varyings;
  const float* constants;              /* the pixel shader's SG_MAX_SHADER_CONSTANTS */
  void* backend;
  void (*ddx)(void* backend, uint32_t reg, float out[4]);
  void (*ddy)(void* backend, uint32_t reg, float out[4]);
  void (*tex2d)(void* backend, uint32_t reg, float out[4]);
  void (*tex2dlod)(void* backend, uint32_t reg, float out[4]);
  void (*tex2dproj)(void* backend, uint32_t reg, float out[4]);
  void (*sample)(void* backend, float u, float v, float lod, float out[4]);  /* sampler::sample */
  void (*sample_grad)(void* backend, float u, float v, float dxu, float dxv, float dyu, float dyv,
                      float out[4]);   /* sampler::sample_2d_grad */
  void (*sample_cube)(void* backend, float x, float y, float z, float lod, float out[4]); /* sampler::sample_cube */
  float color[SG_MAX_COLOR_TARGETS][4]; /* out: ps_output::color */
} sg_host_ps_io;

/* What a host backend hands a blend-shader body for one sample
 * (cpp_blend_shader::execute, shader.cpp:524-526). */
typedef struct sg_host_bs_io {
  uint32_t sample;
  float in_color[SG_MAX_COLOR_TARGETS][4]; /* ps_output::color */
  const float* constants;              /* the blend shader's SG_MAX_SHADER_CONSTANTS */
  void* backend;
  /* pixel_accessor::color(target, sample) and color(target, sample, c) */
  void (*get)(void* backend, uint32_t target, uint32_t sample, float out[4]);
  void (*set)(void* backend, uint32_t target, uint32_t sample, const float c[4]);
} sg_host_bs_io;

typedef struct sg_shader_module {
  uint32_t abi_version;                /* SG_SHADER_ABI_VERSION */
  uint32_t stage;                      /* SG_STAGE_VERTEX, SG_STAGE_PIXEL or SG_STAGE_BLEND */
  const char* name;
  /* Called by a GPU device at registration, its CUDA device current:
   * prepares the module's kernels there (the sampler's weight table of
   * 256 floats, shared-memory limits); 0 on success. */
  int32_t (*device_init)(const float* ewa_table, void* cuda_stream);
  /* Launches the module's kernel for one pass: `pass` is the library's pass
   * parameter block (opaque here), `key` the shade key of the module's
   * fragments (pixel stage) or 0 (blend stage: the pass's merge; vertex
   * stage: the pass's geometry, every draw of the pass). */
  void (*device_launch)(const void* pass, uint32_t key, uint32_t grid, void* cuda_stream);
  /* The body compiled for the host: shader_prog's result (0 discards). */
  int32_t (*host_ps)(sg_host_ps_io* io);
  int32_t (*host_bs)(sg_host_bs_io* io);
  int32_t (*host_vs)(sg_host_vs_io* io);
} sg_shader_module;

/* ---- descriptors ------------------------------------------------------------ */
typedef struct sg_viewport {           /* salvia/include/salvia/core/viewport.h */
  float x, y, w, h, minz, maxz;
} sg_viewport;

typedef struct sg_raster_desc {        /* raster_state.h:17-40 */
  uint32_t fill_mode;                  /* SG_FILL_SOLID, or SG_FILL_WIREFRAME for triangle topologies */
  uint32_t cull_mode;                  /* SG_CULL_* */
  uint32_t front_ccw;
  uint32_t reserved;
} sg_raster_desc;

typedef struct sg_stencil_face_desc {  /* framebuffer.h:20-33 */
  uint32_t fail_op, depth_fail_op, pass_op, func;
} sg_stencil_face_desc;

typedef struct sg_depth_stencil_desc { /* framebuffer.h:35-52 */
  uint32_t depth_enable;
  uint32_t depth_write;
  uint32_t depth_func;
  uint32_t stencil_enable;
  uint32_t stencil_read_mask;          /* low 8 bits used (uint8_t in the reference) */
  uint32_t stencil_write_mask;         /* low 8 bits used */
  sg_stencil_face_desc front, back;
} sg_depth_stencil_desc;

typedef struct sg_sampler_desc {       /* sampler.h:16-45 */
  uint32_t min_filter, mag_filter, mip_filter, mip_quality;
  uint32_t address_u, address_v, address_w;
  uint32_t max_anisotropy;
  float lod_bias;
  float border_color[4];
  float min_lod, max_lod;
} sg_sampler_desc;

typedef struct sg_vertex_stream {      /* set_vertex_buffers (renderer.h:66-70) */
  uint32_t buffer;
  uint32_t stride;
  uint32_t offset;
} sg_vertex_stream;

typedef struct sg_vs_input {           /* input_element_desc (input_layout.h:20-47) bound to a register */
  uint32_t semantic;                   /* SG_SEMANTIC_* */
  uint32_t semantic_index;
  uint32_t format;                     /* SG_VFMT_* */
  uint32_t slot;
  uint32_t offset;                     /* aligned_byte_offset */
} sg_vs_input;

typedef struct sg_shader {
  uint32_t program;                    /* SG_VS_* / SG_PS_* / SG_BS_* */
  uint32_t samplers[SG_MAX_SHADER_SAMPLERS];
  uint32_t learned_filter;             /* SG_PS_TEX_GRAD_LEARNED: sg_af_model_id, else 0 */
  float constants[SG_MAX_SHADER_CONSTANTS];
} sg_shader;

/* One draw / draw_index call with the state it runs under
 * (render_state, salvia/include/salvia/core/render_state.h:46-94). */
typedef struct sg_draw_desc {
  uint32_t color_target;               /* texture handle (level 0), 0 = none */
  uint32_t ds_target;                  /* texture handle, 0 = none */
  sg_viewport viewport;
  uint32_t topology;
  uint32_t indexed;                    /* 0: draw(start, count), 1: draw_index(start, count, base) */
  uint32_t index_buffer;
  uint32_t index_format;
  uint32_t start;
  uint32_t prim_count;
  int32_t base_vertex;                 /* draw_index only: draw() has none (renderer_impl.cpp:337-344) */
  uint32_t num_streams;
  sg_vertex_stream streams[SG_MAX_STREAMS];
  uint32_t num_inputs;
  sg_vs_input inputs[SG_MAX_VS_INPUTS];
  uint32_t num_varyings;               /* cpp_vertex_shader::num_output_attributes */
  uint32_t varying_modifiers[SG_MAX_VARYINGS];
  sg_raster_desc raster;
  sg_depth_stencil_desc depth_stencil;
  int32_t stencil_ref;
  sg_shader vs, ps, bs;
  /* colour targets 1..6 after color_target (0 = none, from the first 0 on):
   * the draw renders into every one; the render area is the smallest of
   * their sizes, as in renderer_impl::set_render_targets, and all have the
   * sample count of color_target */
  uint32_t more_color_targets[SG_MAX_COLOR_TARGETS - 1];
} sg_draw_desc;

/* Pipeline counters of one draw (async_object.h:90-175). */
typedef struct sg_draw_stats {
  uint64_t ia_primitives;              /* input primitives */
  uint64_t cprimitives;                /* triangles after clipping and culling (lines: segments drawn) */
  uint64_t ps_invocations;             /* pixel-shader invocations, helpers included */
  uint64_t backend_input_pixels;       /* pixels of quads that reached the output merger */
  /* vertices the input assembler fetched: three per primitive for lists and
   * strips alike, as the reference's vertex cache counts them
   * (default_vertex_cache.cpp:363) */
  uint64_t ia_vertices;
  /* vertex-shader executions: here one per primitive corner (no vertex
   * reuse across primitives), counted on the device.  The reference counts
   * the misses of its per-thread vertex caches (default_vertex_cache.cpp:
   * 354-400), which depends on how its worker threads split the draw, so
   * this counter is not compared with it. */
  uint64_t vs_invocations;
  /* primitives that entered the clipper: every input primitive
   * (geom_setup_engine.cpp:108-123) */
  uint64_t cinvocations;
} sg_draw_stats;

/* Per-stage device time and launch counts, accumulated while profiling is
 * enabled (the pipeline_profiles query, async_object.h:177-233): geometry
 * covers the reference's vtx_proc/clipping/compact_clip/vp_trans stages,
 * binning its tri_dispatch stage, raster its ras stage.  Times come from
 * CUDA events recorded on the device's stream around each stage; the
 * reference's ras stage is split into cover, shade and merge here. */
typedef struct sg_profile_data {
  double geometry_ms;
  double binning_ms;
  double raster_ms;           /* cover + shade + merge */
  double cover_ms;            /* coverage + early-Z */
  double shade_ms;            /* attribute interpolation + pixel shader */
  double merge_ms;            /* depth-stencil + blend */
  uint64_t draws;
  uint64_t launches;          /* kernels launched (all stages, clears, resolves) */
  uint64_t raster_launches;
  uint64_t af_lookups;        /* lookups the learned filter took */
  uint64_t af_fallbacks;      /* of those, the ones it sent back to the plain sampler */
  uint64_t cover_batches;     /* coverage work: staged triangle batches, */
  uint64_t cover_rounds;      /* walk rounds, */
  uint64_t cover_pairs;       /* and (triangle, 4x4 block) pairs past the hierarchical depth test */
} sg_profile_data;

/* ---- device (create_benchmark_renderer, renderer.h:133-134) --------------- */
typedef struct sg_device sg_device;

/* Creates a device on CUDA device `cuda_device`, issuing all work on
 * `cuda_stream` (a cudaStream_t, or NULL for a stream the device owns). */
int32_t sg_device_create(int32_t cuda_device, void* cuda_stream, sg_device** out_device);
void sg_device_destroy(sg_device* dev);
/* renderer::flush (renderer.h:128): waits until all submitted work is done. */
int32_t sg_sync(sg_device* dev);
/* Last CUDA error text seen by the device (empty when none). */
const char* sg_last_error(sg_device* dev);
/* Starts (enable != 0) or stops per-stage timing and resets the counters
 * (renderer::begin/end on a pipeline_profiles query, renderer.h:116-119). */
int32_t sg_profile_enable(sg_device* dev, int32_t enable);
/* Waits for the device and returns the accumulated profile
 * (renderer::get_data, renderer.h:118). */
int32_t sg_profile_read(sg_device* dev, sg_profile_data* out);

/* ---- buffers (create_buffer + map/unmap, renderer.h:45,61-63) -------------- */
int32_t sg_buffer_create(sg_device* dev, size_t size, uint32_t* out_buffer);
int32_t sg_buffer_upload(sg_device* dev, uint32_t buffer, size_t offset, const void* src, size_t size);
int32_t sg_buffer_download(sg_device* dev, uint32_t buffer, size_t offset, void* dst, size_t size);
int32_t sg_buffer_destroy(sg_device* dev, uint32_t buffer);

/* ---- textures / surfaces (create_tex2d, texture.h, surface.h) ---------------
 * Level 0 of a texture is the surface a render target names.  Texel storage
 * matches surface.cpp:277-295: ((y * w + x) * samples + s) * elem_size. */
int32_t sg_texture_create(sg_device* dev, uint32_t width, uint32_t height, uint32_t samples,
                          uint32_t format, uint32_t* out_texture);
/* renderer::create_texcube (renderer_impl.cpp:250-252): a texture_cube of
 * six faces (texture.h:91-102), subresource `face` for cubemap_faces +x, -x,
 * +y, -y, +z, -z (constants.h:118-125) -- the `level` of upload, download
 * and info.  The reference leaves a cube's LOD range at [0, 0]: lookups read
 * level 0, and sg_texture_gen_mipmap refuses a cube texture
 * (texture_cube::gen_mipmap, texture_cube.cpp:18-30, reads a size it never
 * set). */
int32_t sg_texture_create_cube(sg_device* dev, uint32_t width, uint32_t height, uint32_t samples, uint32_t format,
                               uint32_t* out_texture);
int32_t sg_texture_upload(sg_device* dev, uint32_t texture, uint32_t level, const void* src, size_t size);
int32_t sg_texture_download(sg_device* dev, uint32_t texture, uint32_t level, void* dst, size_t size);
/* texture_2d::gen_mipmap(filter, true) (texture2d.cpp:25-36). */
int32_t sg_texture_gen_mipmap(sg_device* dev, uint32_t texture, uint32_t filter);
int32_t sg_texture_info(sg_device* dev, uint32_t texture, uint32_t level, uint32_t* width,
                        uint32_t* height, uint32_t* samples, uint32_t* format, uint32_t* levels);
int32_t sg_texture_destroy(sg_device* dev, uint32_t texture);

/* ---- image ingest and export (salvia/src/ext/resource/texture/tex_io.cpp) ---
 * The reference decodes with FreeImage (load_image, freeimage_utility.cpp:8-18)
 * and copies the bitmap into a surface (copy_image_to_surface_impl,
 * tex_io.cpp:27-53).  Here a project-written PNG decoder stands in for
 * FreeImage; an sg_image is the bitmap as copy_image_to_surface reads it:
 * FreeImage's scanline order (row 0 is the image's BOTTOM line), R, G, B[, A]
 * bytes per pixel, no padding.
 *
 * Decodable: PNG, 8 bits per channel, colour type 2 (RGB, FIT_BITMAP 24 bpp)
 * or 6 (RGBA, 32 bpp), interlaced or not -- the bitmaps check_image_type_support
 * (freeimage_utility.cpp:20-50) accepts.  Everything else returns SG_FAILED
 * (the reference's load_texture returns a null texture for 16-bit and float
 * bitmaps and copies garbage from palette and grey ones).  Critical chunks
 * must pass their CRC, the zlib stream its Adler-32, and the image data must
 * fill the image exactly. */
typedef struct sg_image {
  uint32_t width;
  uint32_t height;
  uint32_t channels;  /* 3: RGB (alpha reads 0, tex_io.cpp:29-31,66); 4: RGBA */
  uint32_t reserved;
  uint8_t* pixels;    /* width * height * channels bytes, owned by the library */
} sg_image;
/* A byte string the library allocated (an encoded file). */
typedef struct sg_blob {
  uint8_t* data;
  size_t size;
} sg_blob;
/* load_image: decodes `size` bytes of an image file (host only, no device). */
int32_t sg_image_decode(const void* file, size_t size, sg_image* out);
void sg_image_release(sg_image* image);
void sg_blob_release(sg_blob* blob);
/* copy_image_to_surface (tex_io.cpp:27-74): converts the image into level
 * `level` (a cube face for a cube texture) of a 1-sample colour texture of
 * the same size, each pixel color_rgba8 -> the texture's format
 * (pixel_format_convertor, color_convertors.cpp), on the device. */
int32_t sg_texture_write_image(sg_device* dev, uint32_t texture, uint32_t level, const sg_image* image);
/* save_surface (tex_io.cpp:139-188): encodes level `level` of a 1-sample
 * colour texture as a PNG (image_format SG_FMT_BGRA8: 8-bit RGBA) or a
 * Radiance RGBE file (SG_FMT_RGB32F), rows in FreeImage's order (the file's
 * top line is the surface's last row).  Other formats: SG_INVALID_PARAMETER
 * (the reference stops at ef_unimplemented). */
int32_t sg_texture_encode_image(sg_device* dev, uint32_t texture, uint32_t level, uint32_t image_format,
                                sg_blob* out);
/* The host encoders behind sg_texture_encode_image: `image` rows in
 * FreeImage's order (row 0 is written as the file's last line).  PNG: 3 or 4
 * channels.  HDR: `rgb` holds width * height * 3 floats. */
int32_t sg_image_encode_png(const sg_image* image, sg_blob* out);
int32_t sg_image_encode_hdr(const float* rgb, uint32_t width, uint32_t height, sg_blob* out);

/* ---- mesh ingest (salvia/src/ext/resource/mesh/mesh_io_obj.cpp) ------------
 * create_mesh_from_obj (mesh_io_obj.cpp:436-455): parses a Wavefront OBJ file
 * as load_obj_mesh_c does (mesh_io_obj.cpp:140-263: v / vt / vn / f with the
 * first three corners of each face, usemtl, mtllib, vertices shared by
 * (position, texcoord, normal) index triple, the rest of each line skipped)
 * and its material library as load_material does (mesh_io_obj.cpp:59-138),
 * then splits the faces per material as construct_meshes does
 * (mesh_io_obj.cpp:375-434).  One sg_obj_material per mesh the reference
 * returns: the materials with at least one face, in material order.  An index
 * outside its array (the reference reads out of bounds) or a token longer
 * than the reference's 2048-byte buffer returns SG_FAILED. */
typedef struct sg_obj_material {
  const char* name;       /* obj_material::name ("default" for material 0) */
  const char* tex_name;   /* map_Kd with '\\' replaced by '/' ("" when none) */
  const char* tex_path;   /* tex_name against the OBJ file's directory ("" when none) */
  float ambient[4];
  float diffuse[4];
  float specular[4];
  int32_t shininess;
  float alpha;
  int32_t is_specular;
  uint32_t first_index;   /* this mesh's triangles: indices[first_index, first_index + index_count) */
  uint32_t index_count;
  uint32_t reserved;
} sg_obj_material;
typedef struct sg_obj_mesh {
  uint32_t num_vertices;
  uint32_t num_indices;
  uint32_t num_materials;
  uint32_t reserved;
  const float* vertices;   /* obj_mesh_vertex: position, texcoord, normal, 4 floats each */
  const uint32_t* indices; /* format_r32_uint, grouped by material */
  const sg_obj_material* materials;
} sg_obj_mesh;
int32_t sg_obj_load(const char* path, int32_t flip_tex_v, sg_obj_mesh** out);
void sg_obj_release(sg_obj_mesh* mesh);

/* ---- SASL shaders -------------------------------------------------------------
 * renderer.h:136-147 compile(code, lang) runs the reference's SASL compiler
 * (an LLVM JIT) on a vertex or pixel shader.  sg_sasl_translate turns the
 * same source into the C++ class of a user shader module: the text of a
 * translation unit that includes <salvia_gb300/sasl_rt.cuh> and exports
 * salvia_gb300_module_<class_name>(), to be built with nvcc (the GPU module)
 * or a host C++ compiler (the host body alone).  `language` is the
 * reference's languages value (constants.h:11-20); `entry` names the entry
 * function (NULL: main, vs_main or ps_main, else the last function).  The
 * reflection text lists the stage interface one item a line ("input
 * SEMANTIC INDEX REGISTER COMPONENTS", "output ...", "uniform NAME WORD
 * WORDS BASE ROWS COLS", "sampler NAME SLOT", "varyings N", "words N").
 * Returns SG_INVALID_PARAMETER with the message in *out_log when the source
 * does not translate; the strings are freed with sg_sasl_free. */
enum { SG_LANG_GENERAL = 1, SG_LANG_VERTEX_SHADER = 2, SG_LANG_PIXEL_SHADER = 3, SG_LANG_BLENDING_SHADER = 4 };
int32_t sg_sasl_translate(const char* source, uint32_t language, const char* entry, const char* class_name,
                          char** out_source, char** out_reflection, char** out_log);
void sg_sasl_free(char* p);

/* ---- samplers (create_sampler, renderer.h:49) ------------------------------- */
int32_t sg_sampler_create(sg_device* dev, const sg_sampler_desc* desc, uint32_t texture,
                          uint32_t* out_sampler);
int32_t sg_sampler_destroy(sg_device* dev, uint32_t sampler);

/* ---- commands --------------------------------------------------------------- */
/* renderer::draw / draw_index (renderer.h:121-122).  `stats` may be NULL;
 * when given, the counters are written once the draw has completed on the
 * device (the call then synchronises). */
int32_t sg_draw(sg_device* dev, const sg_draw_desc* desc, sg_draw_stats* stats);

/* Size of the static scratch used by sg_draw_static_scratch, per CUDA device. */
#define SG_STATIC_SCRATCH_BYTES (64u << 20)
/* Part of it that the draw-sized tables may take (see below). */
#define SG_STATIC_SCRATCH_TABLE_LIMIT (48u << 20)

/* sg_draw that allocates nothing: no counterpart in the reference.
 *
 * Same pipeline, kernels and results as sg_draw, but every per-draw scratch
 * buffer (triangle records, bin counters and entries, fragment chunks, tile
 * tables, draw counters) is carved from one file-scope device array of
 * SG_STATIC_SCRATCH_BYTES instead of the device's grow-only arenas, and no
 * profiling events are taken.  It serves callers that must not allocate
 * device memory during a frame: a host whose device memory is budgeted by
 * another allocator (a pre-reserved pool that a cudaMalloc would go around
 * or fail against), and frame loops that cannot take the device-wide
 * synchronisation of the cudaFree/cudaMalloc pair an arena grows with.
 *
 * Limits: the draw-sized tables (the draw's parameter block, 3 slots per
 * primitive of 4 + 16 * (8 + 3 * num_varyings) bytes, tiles x bin chunks
 * counters, 1 KiB per 64x64 tile) must fit in
 * SG_STATIC_SCRATCH_TABLE_LIMIT; a larger draw is rejected with
 * SG_INVALID_PARAMETER and a message in sg_last_error before any kernel is
 * launched.  Bin entries and fragment chunks share the rest; a draw whose
 * coverage needs more returns SG_OUT_OF_MEMORY (with `stats`; otherwise at
 * the next sg_sync) and leaves its targets partly drawn, as sg_draw does on
 * an overflow.
 *
 * The first call on each CUDA device does setup: the device's module is
 * loaded and the array's address looked up (cudaGetSymbolAddress) with that
 * device current; make that first call before any stream capture.  Only the
 * draw counters must start at zero, and the call clears them on its stream.
 * All callers on one CUDA device share the array: calls whose work may
 * overlap on the device (other sg_device handles, other streams) race and
 * must be ordered by the caller; calls through one handle are ordered by
 * its stream. */
int32_t sg_draw_static_scratch(sg_device* dev, const sg_draw_desc* desc, sg_draw_stats* stats);

/* ---- batched submission --------------------------------------------------
 * A command list of draws, clears and resolves, possibly over many render
 * targets (many frames).  Results are exactly those of issuing the commands
 * one by one through sg_draw / sg_clear_* / sg_resolve (the reference
 * executes render_core commands in order, render_core.cpp:30-61); the
 * runtime groups them into passes, each pass one kernel chain over all of
 * its draws and targets, splitting where order matters: a target cleared,
 * resolved or sampled between two of its draws, a draw whose depth test runs
 * before shading (no stencil) after one whose test runs after shading on the
 * same depth target, or a pass reaching SG_PASS_MAX_PRIMS primitives or
 * SG_PASS_MAX_SAMPLES target samples. */
enum { SG_CMD_DRAW = 1, SG_CMD_CLEAR_COLOR = 2, SG_CMD_CLEAR_DEPTH_STENCIL = 3, SG_CMD_RESOLVE = 4 };
#define SG_PASS_MAX_PRIMS (1u << 24)
#define SG_PASS_MAX_SAMPLES (1ull << 26)

typedef struct sg_command {
  uint32_t type;                       /* SG_CMD_* */
  uint32_t texture;                    /* clear target; resolve source */
  uint32_t texture2;                   /* resolve destination */
  uint32_t flags;                      /* SG_CLEAR_DEPTH | SG_CLEAR_STENCIL */
  float color[4];                      /* clear colour */
  float depth;
  uint32_t stencil;
  const sg_draw_desc* draw;            /* SG_CMD_DRAW */
} sg_command;

/* Executes `n` commands in order.  `stats` may be NULL, else it holds one
 * entry per command (zero for non-draw commands) and the call synchronises. */
int32_t sg_submit(sg_device* dev, const sg_command* cmds, uint32_t n, sg_draw_stats* stats);

/* Recorded command lists: no counterpart in the reference (its async
 * renderer queues commands to a render thread, async_renderer.cpp:19-104;
 * here a list becomes one CUDA graph).  sg_graph_create executes the list
 * once (exactly as sg_submit would, so the targets hold one execution's
 * results), sizes private scratch for it from that run's counters, and
 * captures every pass into one CUDA graph with the draw parameters resident
 * on the device.  sg_graph_launch replays the whole list as one graph
 * launch on the device's stream; the buffers, textures and samplers the
 * list names must stay alive and keep their sizes.  Replays of the same
 * inputs need the same scratch; a replay whose inputs changed so much that
 * the scratch overflows reports SG_OUT_OF_MEMORY at the next sg_sync. */
typedef struct sg_graph sg_graph;
int32_t sg_graph_create(sg_device* dev, const sg_command* cmds, uint32_t n, sg_graph** out_graph);
int32_t sg_graph_launch(sg_device* dev, sg_graph* graph);
/* Launches of the graph recorded so far and the passes it holds. */
int32_t sg_graph_info(sg_device* dev, sg_graph* graph, uint32_t* passes, uint32_t* kernels);
void sg_graph_destroy(sg_device* dev, sg_graph* graph);

/* ---- scheduling parameters and the autotuner ------------------------------
 * None of these changes results, only how the work is cut: the coverage
 * work-item edge (16 or 32 pixels; a 64x64 binning tile is covered as four
 * 32x32 items or sixteen 16x16 items, the latter also for any tile with more
 * than `split_entries` bin entries), the minimum triangle slots per binning
 * warp, the initial bin-entry and fragment capacities, the pixel-shading
 * quads per warp, CTAs per SM for the shading and merging kernels, and the
 * threads that cover one 4x4 block: 2 (each half of its samples, walking the
 * block's triangles in order; 32x32 items) or 32 (a warp per triangle-block
 * pair, the `cover_item` and `split_entries` choices apply). */
typedef struct sg_tuning {
  uint32_t cover_item;       /* 16 or 32 */
  uint32_t split_entries;    /* 32x32 items become 16x16 above this many bin entries */
  uint32_t bin_chunk;        /* slots per binning warp, power of two >= 64 */
  uint32_t bin_capacity;     /* initial bin entries */
  uint32_t frag_chunks;      /* initial fragment chunks (16 quads each) */
  uint32_t shade_quads_per_warp; /* 8 (4 lanes per quad) */
  uint32_t shade_ctas_per_sm;
  uint32_t merge_ctas_per_sm;
  uint32_t cover_threads_per_block; /* 2 or 32 */
  uint32_t cover_ctas_per_sm;  /* 3 or 4: the 2-thread coverage kernel's registers cut for that many CTAs per SM */
  uint32_t shade_resident;     /* 3 or 4: the shading kernels' registers cut for that many CTAs per SM */
  uint32_t merge_resident;     /* 3 or 4: the merging kernel's registers cut for that many CTAs per SM */
} sg_tuning;
int32_t sg_get_tuning(sg_device* dev, sg_tuning* out);
int32_t sg_set_tuning(sg_device* dev, const sg_tuning* tuning);
/* Times the command list under candidate tunings (CUDA events on the
 * device's stream, `reps` runs each after one warm-up) and keeps the fastest
 * in the device; `out` receives it and `best_ms` its time (either may be
 * NULL).  The targets hold the last run's results, identical for every
 * candidate. */
int32_t sg_autotune(sg_device* dev, const sg_command* cmds, uint32_t n, uint32_t reps, sg_tuning* out,
                    float* best_ms);
/* The autotuner's search space, in the order it searches (coordinate
 * descent, two sweeps): each searched sg_tuning field by name with its
 * candidate values.  Not searched: the binning tile (64x64 by the reference's
 * classification), shade_quads_per_warp (8 by construction), and the
 * capacities (sized from counters and grown after an overflow). */
typedef struct sg_tuning_knob {
  const char* field;
  uint32_t count;
  uint32_t values[8];
} sg_tuning_knob;
int32_t sg_autotune_space(const sg_tuning_knob** knobs, uint32_t* count);

/* ---- learned anisotropic filter --------------------------------------------
 * No counterpart in the reference.  A small MLP (24 inputs -> 64 -> 64 -> 5,
 * GELU in its tanh form, BF16 weights and activations, FP32 accumulate on the
 * tensor cores) that predicts sampler::sample_2d_grad's anisotropic result
 * and a confidence from the texel-space derivatives, the anisotropy measures
 * of calc_anisotropic_info and four bilinear taps along the major axis
 * (sampler.cpp:730-760,875-958).  Features, in order: the two derivatives in
 * texels divided by the longer one's length (4), the probes' mip level / 8,
 * log2 of the longer derivative's length / 8, the probe count / 16, log2 of
 * the anisotropy ratio / 4, and the RGBA of bilinear taps at the probes'
 * level at -3/8, -1/8, 1/8 and 3/8 of the probe span (16).  The predicted
 * colour is 0.25 * ((tap0 + tap1) + (tap2 + tap3)) (float32) plus the
 * network's first four outputs; the confidence is the sigmoid of the fifth.
 * Parameters are fp32 masters in the order W1 [64 x 24], b1 [64],
 * W2 [64 x 64], b2 [64], W3 [5 x 64], b3 [5] (W[out][in]). */
#define SG_AF_FEATURES 24
#define SG_AF_OUTPUTS 5
#define SG_AF_PARAMS 6085
typedef struct sg_af_model sg_af_model;
/* Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights from `seed`, zero biases. */
int32_t sg_af_model_create(sg_device* dev, uint64_t seed, sg_af_model** out_model);
/* Destroy recorded graphs that draw with the model before the model. */
void sg_af_model_destroy(sg_device* dev, sg_af_model* model);
/* The id a pixel shader names the model by (sg_shader.learned_filter). */
uint32_t sg_af_model_id(const sg_af_model* model);
int32_t sg_af_model_get_params(sg_device* dev, sg_af_model* model, float* params /* SG_AF_PARAMS */);
int32_t sg_af_model_set_params(sg_device* dev, sg_af_model* model, const float* params);
/* Inference on the tensor cores: `features` n x 24 (the network reads them
 * rounded to BF16), `out` n x 5 (predicted RGBA, confidence in [0, 1]). */
int32_t sg_af_model_forward(sg_device* dev, sg_af_model* model, const float* features, uint32_t n, float* out);
/* Draws n random anisotropic lookups on the samplers (lookup i on sampler
 * i mod num_samplers: uniform position, minor axis 2^U(0, 7) texels, ratio
 * U(2.5, 16), major axis at a uniform angle) and writes their features
 * (n x 24) and the plain sampler's result as the target (n x 4 RGBA). */
int32_t sg_af_sample(sg_device* dev, const uint32_t* samplers, uint32_t num_samplers, uint32_t n, uint64_t seed,
                     float* features, float* targets);
/* One forward and backward pass on the tensor cores over n samples: `grads`
 * (SG_AF_PARAMS) receives the gradient of the mean loss, `loss` the mean
 * loss.  Loss of one sample: the squared error of the predicted colour plus
 * the binary cross-entropy of the confidence against
 * exp(-32 * max |colour error|).  The parameters do not change. */
int32_t sg_af_model_gradients(sg_device* dev, sg_af_model* model, const float* features, const float* targets,
                              uint32_t n, float* grads, float* loss);
/* Creates `count` tileable RGBA8 textures of size x size (a power of two,
 * 16-4096) with full box-filtered mip chains, filled on the device from
 * `seed`: texture i is value noise (4-8 octaves from 2, 4 or 8 cells) when
 * i mod 3 == 0, a two-colour checkerboard with a period of 2-64 texels when
 * i mod 3 == 1, and an RGBA sinusoidal grating at a random orientation with
 * a period of 2-64 texels when i mod 3 == 2.  The handles go to
 * `out_textures` (count entries); they are ordinary textures. */
int32_t sg_af_make_textures(sg_device* dev, uint32_t count, uint32_t size, uint64_t seed, uint32_t* out_textures);
typedef struct sg_af_train_desc {
  const uint32_t* samplers; /* training textures (sampler handles) */
  uint32_t num_samplers;
  uint32_t samples;         /* training set size, drawn once as sg_af_sample does */
  uint32_t batch;           /* samples per Adam step */
  uint32_t epochs;
  float lr;                 /* Adam step size (beta1 0.9, beta2 0.999, eps 1e-8) */
  uint64_t seed;
} sg_af_train_desc;
typedef struct sg_af_report {
  float first_loss;         /* mean per-sample loss over the first and the last
                               min(16, steps / 4) batches (at least one) */
  float last_loss;
  uint32_t steps;
  float train_ms;           /* device time of the steps (CUDA events) */
} sg_af_report;
/* Trains the model on the device: the training set is sampled from the plain
 * anisotropic sampler, then each step is a tensor-core forward and backward
 * pass over one batch and an Adam update of the fp32 masters. */
int32_t sg_af_model_train(sg_device* dev, sg_af_model* model, const sg_af_train_desc* desc, sg_af_report* report);

/* Registers a user shader module on the device (see sg_shader_module) and
 * returns its program id; the module must outlive the device.  The same
 * module registered twice gets the same id. */
int32_t sg_shader_register(sg_device* dev, const sg_shader_module* module, uint32_t* out_program);

/* renderer::clear_color (renderer.h:124). */
int32_t sg_clear_color(sg_device* dev, uint32_t texture, const float rgba[4]);
/* renderer::clear_depth_stencil (renderer.h:125-126). */
int32_t sg_clear_depth_stencil(sg_device* dev, uint32_t texture, uint32_t flags, float depth,
                               uint32_t stencil);
/* surface::resolve (surface.cpp:123-140): box average of the samples of
 * `src` (level 0) into the single-sample `dst` (level 0). */
int32_t sg_resolve(sg_device* dev, uint32_t src, uint32_t dst);

#ifdef __cplusplus
}
#endif

#endif /* SALVIA_GB300_H */
