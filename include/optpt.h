/* optpt: C ABI of the GB300 progressive path tracer.
 *
 * This is the drop-in boundary for markcmagro/optix_pt's render call. The
 * reference drives rendering through the C++ class Renderer
 * (include/renderer.h:19-206): an init sequence that loads the scene and builds
 * the acceleration structure, then per frame updateLaunchParams() + launch(),
 * then getFrameBuffer(). Each entry point below names the reference member or
 * program it replaces. The C++ Renderer in include/optix_pt/renderer.hpp keeps
 * the reference's method names on top of these calls.
 *
 * Conventions: every function returns an int status (OPTPT_OK or a negative
 * OPTPT_ERR_* code), never throws and never traps; optpt_last_error() gives a
 * message for the last failure on the calling thread. Pointers documented as
 * "device" are CUDA device pointers; "stream" is a cudaStream_t passed as
 * void* (NULL = legacy default stream). One renderer handle must not be used
 * by two host threads at once.
 */
#pragma once
#include <stddef.h>
#include <stdint.h>
#include "optix_pt/launch_params.h"
#include "optix_pt/light.h"
#include "optix_pt/material_data.h"

#ifdef __cplusplus
extern "C" {
#endif

#define OPTPT_OK 0
#define OPTPT_ERR_INVALID (-1)   /* bad argument or size                    */
#define OPTPT_ERR_CUDA (-2)      /* CUDA runtime or kernel launch failure   */
#define OPTPT_ERR_IO (-3)        /* file missing or unreadable              */
#define OPTPT_ERR_PARSE (-4)     /* malformed JSON scene description        */
#define OPTPT_ERR_NOMEM (-5)     /* host or device allocation failed        */
#define OPTPT_ERR_TIMEOUT (-6)   /* a bounded device wait gave up           */
#define OPTPT_ERR_STATE (-7)     /* call out of order (e.g. no framebuffer) */

typedef struct optpt_renderer optpt_renderer;

/* Message for the last failing call on this thread ("" if none). */
const char *optpt_last_error(void);

/* Library version (major * 10000 + minor * 100 + patch). */
int optpt_version(void);

/* ------------------------------------------------------------------ scene */

/* An RGBA8 texture image. wrap: 0 repeat, 1 clamp, 2 mirror. srgb: decode
 * the colour channels from sRGB. filter: 0 bilinear, 1 nearest (the
 * reference's cudaFilterModeLinear / Point, src/renderer.cpp:1471-1530). */
typedef struct optpt_texture {
    uint32_t width;
    uint32_t height;
    const uint8_t *rgba;
    int32_t wrapS;
    int32_t wrapT;
    int32_t srgb;
    int32_t filter;
} optpt_texture;

/* A flattened, world-space triangle scene plus camera and frame settings:
 * what the reference's glTF loader produces (SceneProperties,
 * include/scene_properties.h:11) and SceneDesc adds (include/scene_desc.h:9-39).
 * All arrays are host memory owned by the caller. */
typedef struct optpt_scene {
    const float *positions;     /* float3 per vertex                          */
    uint32_t numVertices;
    const float *normals;       /* float3 per vertex, or NULL                 */
    const float *texCoords;     /* float2 per vertex, or NULL                 */
    const int32_t *triIndices;  /* int3 per triangle                          */
    uint32_t numTriangles;
    const int32_t *matIndices;  /* material per triangle                      */
    const MaterialData *materials;
    uint32_t numMaterials;
    const Light *lights;
    uint32_t numLights;
    const optpt_texture *textures;
    uint32_t numTextures;
    float camEye[3];
    float camTarget[3];
    float camUp[3];
    float camFovYDeg;
    uint32_t resX;
    uint32_t resY;
    float bgColour[3];
    uint32_t spp;               /* samples per pixel the workload asks for    */
    uint32_t maxDepth;
} optpt_scene;

/* Builds one of the seeded procedural scenes into library-owned host arrays
 * (released with optpt_scene_release): "cornell" (36 triangles),
 * "spheres" (8x8 icosphere material sweep, 327,682 triangles).
 * Stands in for the reference's glTF import (src/gltf_loader.cpp:72). */
int optpt_scene_procedural(const char *name, uint32_t seed, optpt_scene *out);
void optpt_scene_release(optpt_scene *scene);

/* Resolves a scene-selection list in the reference's configs/<name>.json format
 * (src/scene_desc.cpp:118-153: {"scene": id, id: name}) and parses the named
 * scene file (src/scene_desc.cpp:50-116). A scene file names either
 * "gltf scene file" (imported with optpt_scene_from_gltf; a relative path is
 * tried against the working directory, as the reference opens it, then
 * against the scene file's directory; "gltf up hint" sets the camera's up
 * vector) or "procedural scene"; "renderer.dimensions" and
 * "renderer.background colour" override the scene's defaults. */
int optpt_scene_from_config(const char *sceneListPath, optpt_scene *out);

/* Imports a glTF 2.0 scene (.gltf with external or data-URI buffers, or a
 * binary .glb) into library-owned host arrays (released with
 * optpt_scene_release), as the reference's GltfLoader::parse/loadScene and
 * Renderer::loadScene/updateScene do (src/gltf_loader.cpp:19-1388,
 * src/renderer.cpp:191-265,1060-1303): the default scene's mesh nodes
 * flattened to world space, materials with KHR_materials_{specular,
 * transmission, ior, emissive_strength, clearcoat, sheen} and
 * KHR_texture_transform, PNG textures decoded to RGBA8, KHR_lights_punctual
 * lights and the first perspective camera; PNG and baseline JPEG images.
 * upHint may be NULL ((0, 1, 0)).
 * Frame defaults: 1280 x 720, 64 spp, depth 8. Errors: OPTPT_ERR_IO for an
 * unreadable file, OPTPT_ERR_PARSE for malformed JSON, buffers or images. */
int optpt_scene_from_gltf(const char *path, const float upHint[3], optpt_scene *out);

/* ------------------------------------------------------------------ animation */

/* A glTF scene kept in memory so that it can be posed at any time: its node
 * tree, skins and one animation (the reference's loadAnimations,
 * src/gltf_loader.cpp:1390-1509: animation 2 when the file has three or
 * more, else 0), evaluated as Renderer::updateScene does each frame
 * (src/renderer.cpp:1060-1303). */
typedef struct optpt_gltf optpt_gltf;

typedef struct optpt_gltf_info_t {
    uint32_t numVertices;   /* of the flattened scene                      */
    uint32_t numShapes;     /* mesh nodes (one matrix slot each)           */
    uint32_t numJointSlots; /* joint matrices over all skinned shapes      */
    uint32_t numChannels;   /* animated translation/rotation/scale targets */
    float duration;         /* last key time of the animation (0: static)  */
    int32_t skinned;
} optpt_gltf_info_t;

/* How each vertex of a renderer's scene follows a pose: rest position (and
 * normal) in its shape's space, the shape's matrix slot and, for skinned
 * vertices, four joint-matrix slots and weights (joints/weights NULL when
 * nothing is skinned). Host arrays. */
typedef struct optpt_deformation {
    const float *restPositions; /* float3 per vertex                        */
    const float *restNormals;   /* float3 per vertex, or NULL               */
    const uint32_t *vertexShape;
    const uint16_t *joints;     /* 4 per vertex, or NULL                    */
    const float *weights;       /* 4 per vertex, or NULL                    */
    uint32_t numVertices;
    uint32_t numShapes;
    uint32_t numJoints;
} optpt_deformation;

int optpt_gltf_open(const char *path, const float upHint[3], optpt_gltf **out);
void optpt_gltf_close(optpt_gltf *g);
int optpt_gltf_info(const optpt_gltf *g, optpt_gltf_info_t *info);
/* The flattened scene at `time` (animate 0: rest pose, no animation), into
 * library-owned arrays released with optpt_scene_release. */
int optpt_gltf_scene(const optpt_gltf *g, float time, int animate, optpt_scene *out);
/* Pointers into the model (valid until optpt_gltf_close). */
int optpt_gltf_deformation(const optpt_gltf *g, optpt_deformation *out);
/* The pose at `time`: per shape its world matrix (16 floats, column-major)
 * and normal matrix (9 floats, row r multiplies the normal: the inverse
 * transpose of the world matrix's 3x3); per joint slot inverse(world(mesh
 * node)) * world(joint) * inverseBind. Any output may be NULL. */
int optpt_gltf_pose(const optpt_gltf *g, float time, float *shapeMatrices, float *shapeNormalMatrices,
                    float *jointMatrices);
/* Positions (and normals, if the scene has them) of every vertex at `time`,
 * on the host, with the same float operations as optpt_deform. */
int optpt_gltf_apply(const optpt_gltf *g, float time, float *positions, float *normals);

/* An RGBA8 image in library-owned memory. */
typedef struct optpt_image {
    uint32_t width;
    uint32_t height;
    uint8_t *rgba;
} optpt_image;

/* Decodes a PNG held in memory to RGBA8 with stb_image's four-component
 * rules (the decoder tinygltf runs for the reference): grey expands to RGB,
 * missing alpha is 255, 16-bit samples keep their high byte, palettes and
 * tRNS apply, Adam7 interlacing is undone. OPTPT_ERR_PARSE on a malformed or
 * truncated file (CRC and Adler-32 checked). */
int optpt_image_decode_png(const void *data, size_t size, optpt_image *out);
/* Decodes a baseline or extended-sequential JPEG (Huffman, 8-bit; grey,
 * YCbCr with any chroma subsampling, Adobe RGB; restart intervals) to RGBA8
 * with alpha 255. Progressive and arithmetic-coded files: OPTPT_ERR_PARSE. */
int optpt_image_decode_jpeg(const void *data, size_t size, optpt_image *out);
void optpt_image_release(optpt_image *img);

/* ------------------------------------------------------------------ renderer */

typedef struct optpt_options {
    uint32_t sppBatch;   /* samples traced side by side in one wavefront (0 = auto) */
    uint32_t blockSize;  /* threads per block for the wavefront kernels (0 = 128)   */
    uint32_t leafSize;   /* maximum triangles per BVH leaf: 1..4 for the 8-wide BVH
                          * (0 = 1), 1..8 for the binary one (0 = 4)                */
    uint32_t useGraph;   /* capture the bounce loop in a CUDA graph (default 1)      */
    uint32_t bvhWidth;   /* 8: compressed 8-wide BVH (default), 2: the binary LBVH   */
    uint32_t compaction; /* queue appends: 0 = auto (one atomic per warp), 32 = per
                          * warp, 1 = per block (one atomic per block and queue)   */
    uint32_t nodeBudget; /* BVH nodes one ray may visit before its walk is cut short
                          * (0 = 2^26, more than any walk of a valid tree needs); a
                          * cut-short walk is counted in optpt_stats               */
    uint32_t tailBounce; /* from this bounce on, one launch finishes every
                          * remaining path (closest hit, shading and shadow rays
                          * per bounce, bit-identical to the per-bounce kernels)
                          * instead of a launch per kernel per bounce; with
                          * guiding on it starts past the guided bounces, at
                          * guiding maxDepth + 1 at the earliest (+ 2 while the
                          * network trains); 0 = OPTPT_DEFAULT_TAIL_BOUNCE,
                          * 0xFFFFFFFF = never                                  */
    uint32_t bvhBuilder; /* binary tree the 8-wide BVH is collapsed from: 0 = the
                          * LBVH (Morton radix tree, reproduced bit for bit by the
                          * host oracle; default), 1 = PLOC clustering on the same
                          * Morton order (leaves of one triangle, leafSize
                          * ignored). The binary BVH (bvhWidth 2) is always the
                          * LBVH.                                                 */
} optpt_options;
#define OPTPT_DEFAULT_TAIL_BOUNCE 5

/* Uploads the scene and builds the BVH on the GPU. Replaces the reference's
 * init sequence Renderer(SceneDesc&) .. loadScene() .. buildAccel(true)
 * (src/renderer.cpp:24,191,267; OptiX context/module/pipeline/SBT set-up has
 * no counterpart). Also performs setupOutputBuffer(resX, resY) and
 * setupCamera() from the scene's camera. `options` may be NULL. */
int optpt_create(const optpt_scene *scene, const optpt_options *options, optpt_renderer **out);
int optpt_destroy(optpt_renderer *r); /* Renderer::~Renderer (src/renderer.cpp:79) */

/* Renderer::setupOutputBuffer (src/renderer.cpp:839): (re)allocates the
 * frame buffers and clears the accumulation. */
int optpt_setup_output_buffer(optpt_renderer *r, uint32_t width, uint32_t height);

/* Renderer::setupCamera + Camera::setupUvwCoordinatSystem
 * (src/renderer.cpp:861, src/camera.cpp:19-40). */
int optpt_setup_camera(optpt_renderer *r, const float eye[3], const float target[3], const float up[3],
                       float fovYDeg);

/* Renderer::setupLaunchParams / updateLaunchParams (src/renderer.cpp:882,910):
 * get returns the current frame contract; set applies sample, seed, eye/U/V/W,
 * vis, tone mapping, gamma, maxDepth and bgColour (buffer pointers, sizes and
 * handles are owned by the renderer and ignored). */
int optpt_get_launch_params(const optpt_renderer *r, LaunchParams *out);
int optpt_set_launch_params(optpt_renderer *r, const LaunchParams *lp);

/* Renders `spp` more samples per pixel into the FP64 accumulation and
 * rewrites frameBuffer / accumFrameBuffer, asynchronously on `stream`.
 * Replaces optixLaunch of __raygen__renderFrame (src/renderer.cpp:943,
 * cu/device_programs.cu:15-106): the reference launches 1 spp per call. */
int optpt_render(optpt_renderer *r, uint32_t spp, void *stream);

/* Renderer::launch (src/renderer.cpp:940-958): 1 spp, wait, copy the
 * tone-mapped frame buffer to the renderer's host buffer. */
int optpt_launch(optpt_renderer *r);

/* Renderer::launch (src/renderer.cpp:940-958) as a pipelined frame loop:
 * renders one frame (1 spp, as optpt_launch), snapshots its tone-mapped
 * frame buffer on the device and copies it to pinned host memory on a copy
 * stream, so the copy overlaps the next frame's rendering instead of
 * following it. *frame receives the previous call's frame, complete in host
 * memory (NULL on the first call after a flush or a resize);
 * optpt_launch_flush waits for the last frame's copy and hands it out. The
 * frames are float4 w*h in two pinned buffers owned by the renderer; one
 * stays valid until the second pipelined call after the one that returned
 * it. Frames are bit-identical to optpt_launch's. */
int optpt_launch_pipelined(optpt_renderer *r, const float **frame);
int optpt_launch_flush(optpt_renderer *r, const float **frame);

/* Renderer::getFrameBuffer (src/renderer.cpp:1344): host float4 w*h owned
 * by the renderer, valid after optpt_launch. NULL before. */
const float *optpt_get_frame_buffer(optpt_renderer *r);

/* Renderer::getSampleCount / resetSampleCount (src/renderer.cpp:1349-1357);
 * reset also clears the accumulation. */
uint32_t optpt_get_sample_count(const optpt_renderer *r);
int optpt_reset_sample_count(optpt_renderer *r);

/* Device pointers of the output buffers (valid until the next
 * optpt_setup_output_buffer): float4 frameBuffer and accumFrameBuffer, and
 * the FP64 per-pixel sums (double4 sum, double4 sum of squares; xyz used). */
int optpt_device_buffers(optpt_renderer *r, float **frameBuffer, float **accumFrameBuffer, double **sum,
                         double **sumSq);

/* Copies the tone-mapped frame buffer (float4 w*h) to caller host memory,
 * ordered on `stream`, and waits for it. */
int optpt_read_frame_buffer(optpt_renderer *r, float *rgbaHost, void *stream);

/* Copies the FP64 per-pixel sums (double4 sum and sum of squares, xyz used,
 * w*h each) to caller host memory, ordered on `stream`, and waits for it. */
int optpt_read_accum(optpt_renderer *r, double *sumHost, double *sumSqHost, void *stream);

/* ------------------------------------------------------------------ scene updates */

/* New vertex positions (and normals, if the scene has them; either may be
 * NULL) as host arrays of the scene's vertex count, then the per-frame work
 * of Renderer::updateScene + updateAccel (src/renderer.cpp:1060-1303): the
 * acceleration structure is refit on the GPU (BVH8: triangle records
 * regathered and every level's quantised boxes recomputed bottom-up, topology
 * kept, as OptiX's update keeps it; the binary BVH is rebuilt), the emissive
 * triangles follow, and accumulation restarts (resetSampleCount). Ordered on
 * `stream`; returns without waiting. */
int optpt_update_vertices(optpt_renderer *r, const float *positions, const float *normals, void *stream);

/* Uploads how the scene's vertices follow a pose (see optpt_deformation and
 * optpt_gltf_deformation); once, before optpt_deform. */
int optpt_set_deformation(optpt_renderer *r, const optpt_deformation *d);

/* Poses the scene on the GPU: uploads the shape matrices (16 floats each),
 * shape normal matrices (9 each) and joint matrices (16 each; NULL when
 * nothing is skinned), deforms every vertex in a kernel with the float
 * operations of optpt_gltf_apply (bit-identical results), then refits as
 * optpt_update_vertices does. Ordered on `stream`. */
int optpt_deform(optpt_renderer *r, const float *shapeMatrices, const float *shapeNormalMatrices,
                 const float *jointMatrices, void *stream);

/* Average CUDA-event time of `reps` back-to-back BVH8 refits of the
 * current vertices (triangle records + every level), for measurement. */
int optpt_refit_profiled(optpt_renderer *r, uint32_t reps, float *msPerRefit);

/* Copies the current vertex positions / normals (either may be NULL) to
 * host memory, ordered on `stream`; waits for it. */
int optpt_read_vertices(optpt_renderer *r, float *positions, float *normals, void *stream);

/* ------------------------------------------------------------------ image output */

/* One GPU pass over the current frame producing the image writers' payloads
 * into caller DEVICE buffers (any may be NULL), ordered on `stream`:
 *   rgba8    w*h uint32: processImage (cu/kernels.cu:22-33) of the tone-mapped
 *            frame buffer, 0xff000000 | r | g << 8 | b << 16 with
 *            r = int(clamp(255.99 x, 0, 255));
 *   rgbe     w*h uint32: Ward RGBE of the accumulated mean radiance (bytes
 *            r, g, b, exponent + 128), as stbi_write_hdr stores it;
 *   halfRows w*h*4 IEEE halves of the accumulated mean with A = 1, each
 *            scanline channel-planar A[w], B[w], G[w], R[w] (an OpenEXR
 *            scanline's layout), rounded to nearest even. */
int optpt_image_out(optpt_renderer *r, uint32_t *rgba8, uint32_t *rgbe, void *halfRows, void *stream);

/* Average CUDA-event time of the output kernel producing all three payloads
 * into library scratch, each of `reps` launches preceded by a 256 MB write
 * that evicts L2 (for roofline measurement). */
int optpt_image_out_profiled(optpt_renderer *r, uint32_t reps, float *msPerLaunch);

/* processImage's RGBA8 copied to caller host memory (w*h uint32, rows top
 * to bottom), ordered on `stream`; waits for it. */
int optpt_read_rgba8(optpt_renderer *r, uint32_t *rgbaHost, void *stream);

/* Writes the current frame to a file, replacing Renderer::dumpFramebuffer,
 * dumpAccumFramebufferRgbe and the EXR dump (src/renderer.cpp:1001-1026,
 * 1361-1370): format 0 PNG (RGBA8 of processImage), 1 Radiance .hdr
 * (run-length encoded RGBE of the accumulated mean), 2 OpenEXR (HALF RGBA of
 * the accumulated mean, A = 1, ZIP compression). path NULL writes the
 * reference's names output.png / output.hdr / output.exr in the working
 * directory. Waits for all GPU work first. */
int optpt_save_image(optpt_renderer *r, int format, const char *path);

/* Host-side encoders for images already in host memory; the encoded file is
 * returned in library-owned memory released with optpt_free.
 *   optpt_encode_png: RGBA8 rows (strideBytes 0 = width * 4);
 *   optpt_encode_hdr: float RGBA pixels to run-length RGBE;
 *   optpt_encode_exr: float RGBA pixels to HALF A, B, G, R with A = 1;
 *                     compression 0 none, 3 ZIP. */
int optpt_encode_png(const uint8_t *rgba, uint32_t width, uint32_t height, size_t strideBytes, void **out,
                     size_t *size);
int optpt_encode_hdr(const float *rgba, uint32_t width, uint32_t height, void **out, size_t *size);
int optpt_encode_exr(const float *rgba, uint32_t width, uint32_t height, int compression, void **out, size_t *size);
void optpt_free(void *p);

/* Counters accumulated since creation (read after the GPU work finished). */
typedef struct optpt_stats {
    uint64_t extensionRays;  /* rays traced by the closest-hit kernel   */
    uint64_t shadowRays;     /* rays traced by the occlusion kernel     */
    uint64_t pathSamples;    /* pixel samples completed                 */
    uint64_t nanSamples;     /* samples dropped for NaN radiance        */
    uint32_t bvhNodes;       /* BVH2 nodes in use                       */
    uint32_t bvhLeaves;
    uint32_t bvh8Nodes;      /* nodes of the compressed 8-wide BVH (0 if not built) */
    uint32_t bvhWidth;       /* BVH traversed: 8 or 2                                */
    uint32_t sppBatch;
    uint32_t blockSize;
    /* Traversal faults, which leave a ray's result possibly wrong and are
     * therefore counted rather than silent (zero on every valid BVH; the
     * reference's OptiX traversal reports none): node groups dropped because
     * a ray's traversal stack was full (binary BVH; the 8-wide BVH's stack
     * cannot overflow, since optpt_create refuses trees deeper than its 64
     * entries), and walks cut short by the node budget
     * (optpt_options.nodeBudget). Rendered and traced rays both count. */
    uint64_t traversalStackOverflows;
    uint64_t traversalBudgetExhausted;
    uint32_t bvh8Levels;     /* levels of the 8-wide BVH (<= 64)                    */
    uint32_t tailBounce;     /* first bounce of plain passes finished by the path-
                              * completion kernel (0: none)                        */
} optpt_stats;
int optpt_get_stats(optpt_renderer *r, optpt_stats *out);

/* Per-kernel device time (ms) of one extra render of `spp` samples, launched
 * without a graph with CUDA events around each kernel on `stream`. Index:
 * 0 generate, 1 extend (closest hit), 2 shade, 3 shadow (occlusion),
 * 4 accumulate + tone map, 5 guiding inference, 6 guiding training (sample
 * gather, gradients, Adam), 7 path completion (the bounces from tailBounce
 * on). Also returns the rays each kernel class traced. */
typedef struct optpt_kernel_times {
    double ms[8];
    uint64_t launches[8];
    uint64_t extensionRays;
    uint64_t shadowRays;
} optpt_kernel_times;
int optpt_render_profiled(optpt_renderer *r, uint32_t spp, void *stream, optpt_kernel_times *out);

/* Queue lengths of the last pass, per bounce d = 1..maxDepth (host arrays of
 * maxDepth entries, any may be NULL): extension rays, point-light and
 * emissive-triangle shadow rays. For relating a profiled launch to the rays
 * it traced; the reference has no counterpart (OptiX hides its queues). */
int optpt_queue_counts(optpt_renderer *r, uint32_t *ext, uint32_t *shadowPoint, uint32_t *shadowEmissive,
                       uint32_t maxDepth);

/* BVH work of one extra render of `spp` samples, run with counting variants
 * of the traversal kernels (slower; not for timing): rays traced, BVH nodes
 * visited and triangles tested, for extension and shadow rays. Feeds the
 * bytes-per-ray model of the traversal roofline. */
typedef struct optpt_traversal_work {
    uint64_t extensionRays;
    uint64_t extensionNodes;
    uint64_t extensionTris;
    uint64_t shadowRays;
    uint64_t shadowNodes;
    uint64_t shadowTris;
} optpt_traversal_work;
int optpt_traversal_counts(optpt_renderer *r, uint32_t spp, void *stream, optpt_traversal_work *out);

/* ------------------------------------------------------------------ error reduction */

/* Relative MSE of a progressive image against a reference image, reduced on
 * the GPU in FP64 (the error measure of the equal-time comparisons; the
 * reference keeps no error metric): mean over pixels of the sum over rgb of
 * (I - R)^2 / (R^2 + 1e-2), with I = sum / nSamples. `sum` and `ref` are
 * device arrays of double4 per pixel (xyz used; an accumulation buffer from
 * optpt_device_buffers and a reference mean image); the result, one double,
 * is written to device memory `out`, ordered on `stream`. Per-tile partial
 * sums (one double per 2048 pixels) are allocated stream-ordered per call. */
int optpt_relmse(const double *sum, uint32_t nSamples, const double *ref, uint32_t numPixels, double *out,
                 void *stream);

/* optpt_relmse for callers that cannot allocate device memory when they call
 * it: a progressive viewer's frame loop that must make no allocator call per
 * frame (cudaMalloc / cudaFree can synchronise the device and stall the
 * frame), or a host application whose own memory pool owns all device memory
 * and forbids a library to allocate behind it. No counterpart in the
 * reference. Same arguments and result; it calls no cudaMalloc, cudaFree or
 * other allocating routine. The partial sums use a fixed 32 KiB array in the
 * library's device memory, which every GPU that loads the library holds until
 * exit; it limits images to 8,388,608 pixels (OPTPT_ERR_INVALID beyond that,
 * before any device work). The first call on a device looks up that array's
 * address (with the device current) and caches it, so make the first call
 * before any stream capture, and do not call it on a device after a
 * cudaDeviceReset (the cached address is then stale). All calls share the
 * array, and each call rewrites every entry it reads: calls that overlap on
 * the GPU (different streams, no ordering) race and must be avoided. */
int optpt_relmse_noalloc(const double *sum, uint32_t nSamples, const double *ref, uint32_t numPixels, double *out,
                         void *stream);

/* ------------------------------------------------------------------ learned guiding network */

/* The path-guiding network (no counterpart in the reference, which samples
 * by the BSDF only): a 16-level hash-grid encoding of position plus the
 * shading normal and outgoing direction, 4 hidden layers of 64 (BF16 on the
 * tensor cores, FP32 accumulation), and 8 von Mises-Fisher lobes out. Created
 * over a world-space box [lo, hi]; parameters initialised from `seed`. */
typedef struct optpt_guide optpt_guide;
int optpt_guide_create(const float lo[3], const float hi[3], uint32_t seed, optpt_guide **out);
int optpt_guide_destroy(optpt_guide *g);

/* Host copies of the FP32 parameters: mlp = 5 x 64 x 64 (W[layer][out][in]),
 * hash = 16 x 2^19 x 2. write = 1 uploads them (and refreshes the BF16 and
 * FP16 working copies), 0 downloads. Either pointer may be NULL. */
int optpt_guide_params(optpt_guide *g, float *mlp, float *hash, int write);

/* The level resolutions, dense-indexing flags and the world -> unit-cube map
 * (u = (p - lo) * invExt), host arrays of 16, 16, 3, 3. */
int optpt_guide_levels(optpt_guide *g, float *res, uint32_t *dense, float *lo, float *invExt);

/* Mixtures for n shading points. Device arrays: queries = 3 float4 each
 * (position, normal, outgoing direction; w ignored); mixtures = 96 bytes
 * each, as halves: per lobe (mu.xyz, kappa), then the 8 weights, then the
 * probability of sampling the mixture rather than the BSDF, then 7 zeros. */
int optpt_guide_infer(optpt_guide *g, const float *queries, uint32_t n, void *mixtures, void *stream);

/* The renderer's own mixture sampler and density (the device functions its
 * shading kernel calls) on n packed mixtures, device arrays in the layout
 * optpt_guide_infer writes. With xi (3 floats per mixture in [0, 1)) each
 * row draws a direction as a guided vertex does (the lobe by xi[0], the
 * direction from it by 1 - xi[1] and xi[2]) and dirPdf (4 floats per row)
 * receives (direction, mixture density there); with xi NULL, dirPdf holds a
 * unit direction per row on input and its 4th float receives the density.
 * Asynchronous on `stream`. */
int optpt_guide_mixture_eval(const void *mixtures, uint32_t n, const float *xi, float *dirPdf, void *stream);

/* Gradient of the batch loss: for the selection probability a (a learned
 * output), sum_i -c_i log(a q(wi_i) + (1 - a) pb_i), the density of the
 * proposal the renderer samples; for the mixture q, sum_i -c_i log q(wi_i)
 * (it learns the whole target). pb_i = the BSDF lobe's density at wi_i,
 * c_i = min(weight_i, 16 * mean positive weight) / sum of weights. The
 * reported loss is the first sum.
 * Device arrays: samples = 4 float4 each ((position, weight), normal,
 * (outgoing, pb), incoming direction wi); *count (device) = samples used,
 * at most `capacity`. Host outputs (NULL to skip): dMlp (5 x 64 x 64), dHash
 * (16 x 2^19 x 2), loss. Synchronises `stream`. */
int optpt_guide_gradients(optpt_guide *g, const float *samples, const uint32_t *count, uint32_t capacity,
                          float *dMlp, float *dHash, double *loss, void *stream);

/* One Adam step (lr 1e-2) on the batch's gradient; asynchronous. */
int optpt_guide_train_step(optpt_guide *g, const float *samples, const uint32_t *count, uint32_t capacity,
                           void *stream);

/* *status = 1 if a tensor-core completion wait expired; the loss and the
 * number of samples of the last training step (either may be NULL). */
int optpt_guide_status(optpt_guide *g, int *status, double *lastLoss, double *lastSamples);

/* ------------------------------------------------------------------ autotuner */

/* Picks the BVH8's binary tree (the LBVH with leaves of up to 1 or 2
 * triangles, or PLOC), the wavefront block size (64, 128, 256)
 * and the shading-queue compaction (per warp, per block) that render the
 * scene fastest (pixel-samples per second) at width x height with `spp`
 * samples timed after `warmupSpp` untimed ones (0 = 2), guiding mode
 * `guiding` (0 plain; see optpt_set_guiding); then, for plain sampling, the
 * tailBounce (never, 3, 4, 5, 6, 8) with those choices. The reference has no
 * counterpart: OptiX makes these choices internally. One renderer per
 * candidate; `trials` (optional) receives every measurement. */
typedef struct optpt_autotune_request {
    uint32_t width;
    uint32_t height;
    uint32_t spp;
    uint32_t warmupSpp;
    uint32_t guiding;
} optpt_autotune_request;
typedef struct optpt_autotune_trial {
    optpt_options options;
    double samplesPerS;
    double mraysPerS;
} optpt_autotune_trial;
int optpt_autotune(const optpt_scene *scene, const optpt_autotune_request *req, optpt_options *best,
                   optpt_autotune_trial *trials, uint32_t maxTrials, uint32_t *numTrials);

/* ------------------------------------------------------------------ batched multi-view */

/* One camera view of the renderer's scene in a batch: a pinhole camera (the
 * reference's Camera, src/camera.cpp:19-40), its resolution and samples. */
typedef struct optpt_view {
    float eye[3];
    float target[3];
    float up[3];
    float fovYDeg;
    uint32_t width;
    uint32_t height;
    uint32_t spp;
    uint32_t scene;  /* optpt_render_batch_scenes: index of the view's renderer
                      * (its scene); ignored by optpt_render_batch */
} optpt_view;

/* Renders every view to its spp in shared wavefront passes (the reference
 * renders one view per launch, src/renderer.cpp:940-1027): the pixels of all
 * views form one queue, each pass gives every unfinished view's pixels the
 * same number of samples (at least 1, about 2^21 paths per pass in all), and
 * the pass is one captured CUDA graph replayed with device-resident sizes.
 * Each view's image equals what a single-view render of that view would
 * estimate; its random streams are keyed by the pixel's index in the batch
 * (view 0 therefore matches a single-view render bit for bit). Guiding, if
 * on, guides and trains on every view. Accumulators restart at each call. */
int optpt_render_batch(optpt_renderer *r, const optpt_view *views, uint32_t numViews, void *stream);

/* Views of several scenes in one batch: renderers[k] holds scene k (its own
 * BVH, materials, lights and guiding network) and view.scene picks the
 * renderer of each view. Every pass is ONE CUDA graph launch whose child
 * graphs are the scenes' captured batch passes, with no dependency between
 * them, so the scenes' bounce loops run side by side on the GPU (a scene
 * whose views are done drops out of the launch). Each renderer's batch holds
 * its own views in the order given: after the call, optpt_batch_view(
 * renderers[k], j, ...) is the j-th view of scene k, bit-identical to the
 * same views rendered by optpt_render_batch on that renderer alone. No
 * counterpart in the reference (one view of one scene per launch). */
int optpt_render_batch_scenes(optpt_renderer *const *renderers, uint32_t numScenes, const optpt_view *views,
                              uint32_t numViews, void *stream);

/* Device pointers into the last batch's buffers for one view: FP64 sums and
 * sums of squares (double4 per pixel, xyz used), the tone-mapped float4
 * frame buffer, and the samples rendered. Valid until the next batch call
 * with a different pixel layout. */
int optpt_batch_view(optpt_renderer *r, uint32_t view, double **sum, double **sumSq, float **frameBuffer,
                     uint32_t *samples);
/* Host copies of one view's FP64 sums and sums of squares (4 doubles per
 * pixel, row-major); either may be NULL. Synchronises `stream`. */
int optpt_batch_read_view(optpt_renderer *r, uint32_t view, double *sumHost, double *sumSqHost, void *stream);

/* Guided sampling in the renderer (replaces nothing in the reference, whose
 * closest-hit program samples the BSDF only, cu/path_tracer.cu:522-581).
 * mode 0: plain BSDF sampling (bit-identical to a renderer that never had
 * guiding); 1: at guidable vertices (non-specular metal, diffuse, rough
 * reflection and coat lobes) the direction comes from the network's mixture
 * with the network's selection probability, else from the BSDF, weighted by
 * the one-sample MIS density; Russian roulette reads the plain estimator's
 * throughput there; the network trains online after every pass on the
 * pass's own radiance estimates; 2: guided sampling with the network frozen.
 * The network is created on first use over the scene's bounding box. */
int optpt_set_guiding(optpt_renderer *r, int mode);
/* Guiding controls (0 / 0.0 fields keep the current value):
 * trainSteps   Adam steps per pass, each on one slice of the pass's samples (4)
 * trainStride  one path in trainStride records training samples (1)
 * maxDepth     vertices up to this depth are guided (all)
 * alphaMin     floor (0) and
 * alphaMax     cap (0.6) on the probability of sampling the network's
 *              mixture instead of the BSDF; between them that probability is
 *              the network's own (a learned output), phased in linearly ...
 * alphaRamp    ... over this many training steps (64)
 * learningRate Adam step size (1e-2)
 * lobeLoss     1: the lobes learn the part of the target the BSDF leaves
 *              (the loss of the whole proposal); 2: the whole target (2);
 *              the selection probability always learns from the loss of the
 *              whole proposal
 * trainSpp     in mode 1, online training stops (the network freezes) once
 *              this many samples per pixel have been rendered with it,
 *              counted from when this value is set or the network created
 *              (0xFFFFFFFF: never stops, the default)
 * primaryShare 1: the first hits of one pixel in a pass share one network
 *              query, its first sample's (the proposal stays exact for every
 *              sample: sampling and density use the same mixture; a quarter
 *              of the inference time on the interior at 320 x 180, but
 *              samples whose first hit lands on another surface than the
 *              first sample's get a worse proposal); -1: one query per
 *              sample, the default. */
typedef struct optpt_guiding_options {
    uint32_t trainSteps;
    uint32_t trainStride;
    uint32_t maxDepth;
    float alphaMin;
    float alphaMax;
    float alphaRamp;
    float learningRate;
    int32_t lobeLoss;
    uint32_t trainSpp;
    int32_t primaryShare;
} optpt_guiding_options;
int optpt_set_guiding_options(optpt_renderer *r, const optpt_guiding_options *o);
int optpt_get_guiding_options(const optpt_renderer *r, optpt_guiding_options *o);

/* The training samples gathered by the last pass (host copy of up to
 * `capacity`, 16 floats each: (position, weight), (normal, -), (outgoing,
 * -), (incoming wi, -)); *count = samples gathered. */
int optpt_guiding_batch(optpt_renderer *r, float *samples, uint32_t capacity, uint32_t *count);

/* The renderer's guiding network (NULL before guiding was first enabled),
 * owned by the renderer. */
int optpt_get_guide(optpt_renderer *r, optpt_guide **out);

/* ------------------------------------------------------------------ tensor-core self-test */

/* Checks this library's tcgen05 operand descriptors and TMEM layouts (no
 * counterpart in the reference, whose OptiX path has no tensor-core code).
 * Device arrays, BF16 bits row-major: A[128][64], B[64][64], G[128][64],
 * X[128][64]. Writes c[128][64] = A B^T (FP32) and dwRaw[128][64] = the TMEM
 * lanes x columns holding G^T X (M = 64); *status = 1 if the MMA completion
 * wait expired. One CTA; asynchronous on `stream`. */
int optpt_tc_selftest(const uint16_t *A, const uint16_t *B, const uint16_t *G, const uint16_t *X, float *c,
                      float *dwRaw, int *status, void *stream);

/* ------------------------------------------------------------------ parity entry points */

/* Closest-hit (anyHit = 0) or occlusion (anyHit = 1) queries against the
 * renderer's BVH, replacing optixTrace (cu/device_programs.cu:63,
 * cu/path_tracer.cu:396,485). Device arrays: rays = 2 float4 per ray
 * (origin.xyz, tmin; direction.xyz, tmax); hits = 1 float4 per ray
 * (t, u, v, primitive index as int bits; -1 = miss). Ties in t resolve to the
 * smaller primitive index. The pixel/sample/depth needed by alpha-blend
 * materials are taken as 0. */
int optpt_trace(optpt_renderer *r, const float *rays, float *hits, uint32_t n, int anyHit, void *stream);

/* The sorted 30-bit Morton codes and the primitive order of the BVH leaves
 * (host copies of numTriangles entries each), and the leaf size used. */
int optpt_bvh_leaf_order(optpt_renderer *r, uint32_t *mortonSorted, int32_t *primOrder);

/* The compressed 8-wide BVH in host memory: `nodes` receives numNodes 80-byte
 * records (layout: optix_pt_gb300/csrc/bvh8.cuh), `primOrder8` the primitive
 * index of every triangle slot in BVH8 leaf order. Either may be NULL to
 * query the count. */
int optpt_bvh8_nodes(optpt_renderer *r, void *nodes, uint32_t capacity, uint32_t *numNodes, int32_t *primOrder8);

/* BVH2 topology in host memory: per node (child0, child1, count0, count1),
 * where count > 0 marks a leaf covering primOrder[child .. child+count). */
int optpt_bvh_nodes(optpt_renderer *r, int32_t *nodes4, uint32_t capacity, uint32_t *numNodes);

/* One BSDF query per element, evaluated by the device BSDF code. Device
 * arrays of optpt_bsdf_query / optpt_bsdf_result (layouts below). The query
 * procedure is the closest-hit program's: categoriseMaterial, the
 * MaterialMetallicRoughness set-up, metallicRoughnessBrdf(l = wi, v = wo),
 * then metallicRoughnessSample with pdf *= categoryWeight
 * (cu/path_tracer.cu:231-370,400,524-526); uniforms are consumed from xs in
 * the reference's draw order. */
typedef struct optpt_bsdf_query {
    float baseColour[3];
    float emission[3];
    float sheenColour[3];
    float metallic;
    float roughness;
    float specular;
    float transmissionWeight;
    float subsurfaceWeight;
    float coatWeight;
    float coatRoughness;
    float sheenRoughnessMat;
    float sheenRoughness;
    float ior;
    uint32_t category;
    float n[3];
    float wo[3];
    float wi[3];
    float xs[12];
} optpt_bsdf_query;

typedef struct optpt_bsdf_result {
    uint32_t category;
    int32_t ret;
    int32_t used;
    float categoryWeight;
    float f[3];
    float dir[3];
    float bsdf[3];
    float pdf;
} optpt_bsdf_result;

int optpt_bsdf_batch(const optpt_bsdf_query *queries, optpt_bsdf_result *results, uint32_t n, void *stream);

#ifdef __cplusplus
}
#endif
