/*
 * gxy_gpu.h -- C ABI of the GB300 ray-processing path (libgxy_gpu.so).
 *
 * Plain C: pointers, sizes and integer status codes; no C++ or torch types.
 * Every entry point returns GXY_OK (0) or a negative GXY_ERR_* code and never
 * throws across the boundary.  Buffers are owned by the caller unless a
 * function name says otherwise.  Entry points are safe to call from several
 * host threads as long as each thread passes its own stream.
 *
 * What each group replaces in Galaxy (paths are inside the Galaxy source tree):
 *
 *   gxy_gpu_trace_raylist       TraceRays::Trace (src/renderer/TraceRays.cpp:68-146), i.e.
 *                               the ISPC exports TraceRays_TraceRays (TraceRays.ispc:326),
 *                               TraceRays_ambientLighting (:735), TraceRays_generateAORays (:625),
 *                               TraceRays_diffuseLighting (:859), TraceRays_generateShadowRays (:763)
 *                               run in the GXY_REVERSE_LIGHTING order (TraceRays.cpp:124-131).
 *   gxy_gpu_classify            Renderer::Classify            (src/renderer/Renderer.cpp:304-421)
 *   gxy_gpu_assign_destinations Renderer::AssignDestinations  (src/renderer/Renderer.cpp:423-454)
 *   gxy_gpu_accumulate_terminated Renderer::HandleTerminatedRays + Rendering::AddLocalPixels
 *                               (src/renderer/Renderer.cpp:456-502, Rendering.cpp:125-153)
 *   gxy_gpu_generate_initial_rays Camera::generate_initial_rays / SpawnRays
 *                               (src/renderer/Camera.cpp:379-493, 528-829) for one partition.
 *   gxy_gpu_scene_commit        Visualization::SetOsprayObjects + Visualization_commit +
 *                               ospCommit(model) (Visualization.cpp:207-285,
 *                               Visualization.ispc:48-93): uploads volumes, transfer
 *                               functions and geometry and builds the BVH on the GPU.
 *   gxy_gpu_render              one frame of Renderer::Start for a RenderingSet
 *                               (Renderer.cpp:179-269, 504-656): ray generation, trace,
 *                               shade, classify, partition hand-off and framebuffer
 *                               accumulation, all on the device.
 */
#ifndef GXY_GPU_H
#define GXY_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define GXY_OK              0
#define GXY_ERR_INVALID    -1   /* bad argument (null pointer, size, count)  */
#define GXY_ERR_CUDA       -2   /* a CUDA runtime call failed                */
#define GXY_ERR_OOM        -3   /* device allocation failed / budget exceeded */
#define GXY_ERR_OVERFLOW   -4   /* a device ray queue overflowed (rays lost)  */
#define GXY_ERR_TIMEOUT    -5   /* a bounded device or host wait ran out      */
#define GXY_ERR_ADMISSION  -6   /* request refused by the HBM budget          */
#define GXY_ERR_NOT_INIT   -7   /* gxy_gpu_init has not been called           */
#define GXY_ERR_CANCELLED  -8   /* the request was cancelled                   */

/* ---- ray flags: src/renderer/RayFlags.h:28-36 -------------------------- */
#define GXY_RAY_PRIMARY    0x001
#define GXY_RAY_SHADOW     0x002
#define GXY_RAY_AO         0x004
#define GXY_RAY_EMPTY      0x008
#define GXY_RAY_SURFACE    0x001
#define GXY_RAY_OPAQUE     0x002
#define GXY_RAY_BOUNDARY   0x004
#define GXY_RAY_TIMEOUT    0x008

/* classifications: src/renderer/Renderer.cpp:78-82 (values >= 0 are partitions) */
#define GXY_TERMINATED     (-1)
#define GXY_DROP_ON_FLOOR  (-2)
#define GXY_KEEP_HERE      (-3)
#define GXY_UNDETERMINED   (-4)

/* light types: src/renderer/Lighting.cpp:58-115, Rendering.cpp:186-200 */
#define GXY_LIGHT_DIRECTIONAL 0
#define GXY_LIGHT_CAMERA      1   /* resolved to GXY_LIGHT_POINT per camera */
#define GXY_LIGHT_POINT       2

#define GXY_TF_SIZE        256
#define GXY_MAX_LIGHTS     8
#define GXY_MAX_SLICES     8
#define GXY_MAX_ISOVALUES  8
#define GXY_MAX_VOLUMES    4
#define GXY_MAX_PARTITIONS 64

/* Transfer function after MappedVis::local_commit (MappedVis.cpp:277-338):
 * 256 resampled RGB entries, 256 resampled opacities and the valueRange. */
typedef struct gxy_tf {
    float colors[GXY_TF_SIZE * 3];
    float opacities[GXY_TF_SIZE];
    float range[2];
} gxy_tf;

/* One VolumeVis over a structured fp32 grid (x fastest).  The grid is the
 * whole dataset; Galaxy's 1-voxel outer ghost shell and brick partition
 * (Volume.cpp:133-172, 379-390) are applied by the scene commit. */
typedef struct gxy_volume_vis {
    const float *samples;
    int32_t counts[3];
    float   origin[3];
    float   deltas[3];
    gxy_tf  tf;
    int32_t n_slices;
    float   slices[GXY_MAX_SLICES][4];        /* plane (nx,ny,nz,d): n.p = d */
    int32_t n_isovalues;
    float   isovalues[GXY_MAX_ISOVALUES];
    int32_t volume_render;
} gxy_volume_vis;

/* TrianglesVis over a triangle mesh (DataDrivenTriangleMesh). */
typedef struct gxy_triangles_vis {
    const float   *vertices;    /* 3 * n_vertices */
    int64_t        n_vertices;
    const int32_t *indices;     /* 3 * n_triangles */
    int64_t        n_triangles;
    const float   *normals;     /* 3 * n_vertices, or NULL (geometric normal) */
    const float   *data;        /* n_vertices, or NULL (white surface)        */
    gxy_tf         tf;
} gxy_triangles_vis;

/* ParticlesVis over spheres (DataDrivenSpheres; radius rules at
 * DataDrivenSpheres.ispc:104-116, ParticlesVis.cpp:104-118). */
typedef struct gxy_particles_vis {
    const float *centers;       /* 3 * n */
    const float *data;          /* n, or NULL */
    int64_t      n;
    float        radius0, radius1, value0, value1;
    gxy_tf       tf;
} gxy_particles_vis;

/* PathLinesVis over polylines (DataDrivenPathLines).  Segment i joins
 * vertices indices[i] and indices[i]+1 (DataDrivenPathLines.cpp:101-104).
 * Per-vertex radius from data by MAP_RADIUS (DataDrivenPathLines.cpp:11-19);
 * a segment is intersected as the capsule of DataDrivenPathLines_intersect_kernel
 * (DataDrivenPathLines.ispc:100-203: cylinder of radius radius0 with a
 * sphere at each end) and coloured as DataDrivenPathLines_postIntersect
 * (DataDrivenPathLines.ispc:213-268: radius interpolated along the segment,
 * mapped back to a data value, looked up in tf). */
typedef struct gxy_pathlines_vis {
    const float   *vertices;    /* 3 * n_vertices */
    const float   *data;        /* n_vertices, or NULL (every radius radius0) */
    int64_t        n_vertices;
    const int32_t *indices;     /* n_segments first-vertex indices */
    int64_t        n_segments;
    float          radius0, radius1, value0, value1;
    gxy_tf         tf;
} gxy_pathlines_vis;

/* Lighting_ispc (Lighting.ih:23-32).  Directional vectors are normalised on
 * load (Lighting.cpp:76-90); camera lights must be resolved first with
 * gxy_resolve_lights. */
typedef struct gxy_lighting {
    int32_t n_lights;
    float   lights[GXY_MAX_LIGHTS][3];
    int32_t types[GXY_MAX_LIGHTS];
    float   Ka, Kd;
    int32_t n_ao;
    float   ao_radius;
    int32_t shadows;
} gxy_lighting;

/* Camera (Camera.h): eye, view direction (not necessarily normalised), up,
 * angle of view in degrees (0 = orthographic) and image size. */
typedef struct gxy_camera {
    float   eye[3];
    float   dir[3];
    float   up[3];
    float   aov;
    int32_t width, height;
} gxy_camera;

/* A Visualization: the scene the tracer consumes. */
typedef struct gxy_scene_desc {
    int32_t                  n_volumes;
    const gxy_volume_vis    *volumes;
    int32_t                  n_triangle_sets;
    const gxy_triangles_vis *triangles;
    int32_t                  n_particle_sets;
    const gxy_particles_vis *particles;
    int32_t partitions[3];   /* brick grid (Galaxy's global_partitions); {1,1,1} = one */
    int32_t has_box;         /* geometry-only scenes: explicit global box below       */
    float   box[6];          /* xmin ymin zmin xmax ymax zmax                          */
    float   sampling_rate;   /* volume samples per voxel; 1.0 in Galaxy                */
    float   opaque_alpha;    /* early-termination alpha; 0.999 in Galaxy               */
    float   epsilon;         /* Renderer.epsilon; 0.001 in Galaxy                      */
    int32_t                  n_pathline_sets;   /* at most 4 */
    const gxy_pathlines_vis *pathlines;
    /* Galaxy partition document (Geometry::get_partitioning, Geometry.cpp:279-350):
     * when n_partition_extents > 0, brick p is partition_extents[6p .. 6p+5] =
     * xmin xmax ymin ymax zmin zmax, face neighbours are found by Galaxy's
     * matching rules, and partitions[] is ignored.  At most 64. */
    int32_t                  n_partition_extents;
    const float             *partition_extents;
} gxy_scene_desc;

/* RayList_ispc (Rays.ih:21-48): 25 SoA arrays plus the count.  Host memory. */
typedef struct gxy_raylist {
    float   *ox, *oy, *oz, *dx, *dy, *dz, *nx, *ny, *nz, *sample;
    float   *r, *g, *b, *o, *sr, *sg, *sb, *so, *t, *tMax;
    int32_t *x, *y, *type, *term, *classification;
    int32_t  n;
} gxy_raylist;

/* Partition geometry as committed (Visualization local/global boxes and
 * neighbours, Visualization.cpp:135-205). */
typedef struct gxy_partition_info {
    float   global_box[6];
    float   local_box[6];
    int32_t neighbors[6];
    int32_t n_partitions;
} gxy_partition_info;

/* Device counters of the last gxy_gpu_render call. */
typedef struct gxy_counters {
    int64_t primary_rays;     /* primary rays generated               */
    int64_t secondary_rays;   /* shadow + AO rays spawned             */
    int64_t shadow_rays;
    int64_t ao_rays;
    int64_t segments;         /* ray x partition traces               */
    int64_t handoffs;         /* rays passed to a neighbour partition */
    int64_t terminated;       /* framebuffer contributions            */
    int64_t dropped;          /* DROP_ON_FLOOR                        */
    int64_t kept;             /* KEEP_HERE re-traces                  */
    int64_t bounces;          /* queue generations processed          */
    int64_t samples;          /* volume samples taken (march positions) */
    int64_t nodes;            /* BVH8 node lines visited              */
    int64_t prim_tests;       /* primitive intersection tests         */
    int32_t overflow;         /* non-zero if a queue overflowed       */
    int32_t bands;            /* bands of image rows the frame was rendered in
                                 (1 unless its queues did not fit at once) */
    int64_t samples_skipped;  /* of `samples`: positions whose voxels were
                                 never read (both ends of their interval in
                                 bricks below the zero-opacity threshold) */
} gxy_counters;

typedef struct gxy_scene_s *gxy_scene;

/* ---- device and scene lifetime ---------------------------------------- */

/* Select the device, cap the bytes this library may allocate (0 = no cap). */
int gxy_gpu_init(int device, size_t hbm_budget_bytes);
int gxy_gpu_shutdown(void);
/* Copy the last error message of this thread into buf. */
int gxy_gpu_last_error(char *buf, int buflen);
/* Bytes currently allocated by the library on the device. */
int gxy_gpu_hbm_in_use(size_t *bytes);

int gxy_gpu_scene_commit(const gxy_scene_desc *desc, gxy_scene *out);
/* Releases one handle (a committed scene or a view); the datasets and the
 * BVH are freed with the last handle that shares them. */
int gxy_gpu_scene_release(gxy_scene scene);

/* Operator kinds of a scene, in gxy_scene_desc order. */
#define GXY_VIS_VOLUME     0
#define GXY_VIS_TRIANGLES  1
#define GXY_VIS_PARTICLES  2
#define GXY_VIS_PATHLINES  3
/* MappedVis_set_transferFunction (src/renderer/MappedVis.ispc:35) after
 * MappedVis::local_commit (MappedVis.cpp:277-338) on a committed scene:
 * replaces the transfer function of operator `index` of kind `vis_kind`.  For
 * a volume the clear-brick flags of the empty-space skipping are recomputed
 * on the device from per-brick bounds kept since the commit; nothing else is
 * rebuilt (no BVH build, no re-bricking).  The work is queued on `stream`
 * (cudaStream_t, NULL = legacy default) and the call returns once it is done,
 * so later frames on any stream see the new function.  Frames of this scene
 * still running on other streams must finish first (the caller orders them;
 * a view, below, avoids the wait).  Frames equal those of a fresh commit with
 * the new function. */
int gxy_gpu_scene_set_tf(gxy_scene scene, int vis_kind, int index, const gxy_tf *tf, void *stream);
/* A new handle on a committed scene, as a second Visualization over the same
 * Datasets (Visualization.cpp:293-340 binds operators to datasets by name):
 * the volumes, geometry and BVH are shared, the transfer functions and the
 * clear-brick flags are the view's own (copies of the scene's current ones).
 * gxy_gpu_scene_set_tf on a view changes only the view, so requests with
 * different transfer functions render concurrently.  Costs the view's
 * transfer-function table, flags and queue counters (a few MiB), no dataset
 * copy.  Release it with gxy_gpu_scene_release. */
int gxy_gpu_scene_view(gxy_scene scene, gxy_scene *out);
int gxy_gpu_scene_partition_info(gxy_scene scene, int partition, gxy_partition_info *out);
/* Host-only: the brick boxes and neighbours a commit of desc would use. */
int gxy_scene_partition_layout(const gxy_scene_desc *desc, int partition, gxy_partition_info *out);
/* BVH statistics: wide nodes, leaf primitive references, build time (ms). */
int gxy_gpu_scene_bvh_info(gxy_scene scene, int64_t *n_nodes, int64_t *n_prim_refs,
                           double *build_ms);

/* Rendering::resolve_lights (Rendering.cpp:157-216): camera-relative lights
 * become point lights for the given camera.  Host-only arithmetic. */
int gxy_resolve_lights(const gxy_lighting *in, const gxy_camera *camera, gxy_lighting *out);

/* ---- whole-frame path (device resident) -------------------------------- */

/* Render one frame of `camera` into the device framebuffer `fb_rgba`
 * (width*height*4 fp32, pixel (x,y) at (y*width+x)*4, y=0 is the bottom row).
 * Contributions are ADDED (Rendering::AddLocalPixels); the caller clears.
 * `stream` is a cudaStream_t (NULL = legacy default stream).  The call is
 * asynchronous with respect to the host except for the per-bounce queue
 * count read-back. */
int gxy_gpu_render(gxy_scene scene, const gxy_camera *camera, const gxy_lighting *lighting,
                   float *fb_rgba, void *stream);
/* Same with a host framebuffer: clears a device framebuffer, renders, copies
 * the image back (the end-to-end call a host application makes). */
int gxy_gpu_render_host(gxy_scene scene, const gxy_camera *camera,
                        const gxy_lighting *lighting, float *host_fb_rgba, void *stream);
int gxy_gpu_query_counters(gxy_scene scene, gxy_counters *out);
/* Per-type primitive test counts and queue records written by the last
 * gxy_gpu_render (inputs of the algorithmic-bytes model). */
int gxy_gpu_query_counters_ex(gxy_scene scene, int64_t *tri_tests, int64_t *sph_tests,
                              int64_t *enqueued);

/* Per-launch statistics of the last gxy_gpu_render, recorded when
 * profiling is on: device time of each kernel launch (CUDA events on the
 * render stream), its generation and kind, and the counters it added. */
typedef struct gxy_generation_stats {
    double  ms;
    int32_t generation;    /* 0 = camera rays                                */
    int32_t kind;          /* 0 camera, 1 primary queue, 2 shadow+AO queues  */
    int64_t rays_in;       /* queue records read (0 for the camera generation) */
    int64_t enqueued;      /* queue records written                         */
    int64_t segments, samples, nodes, tri_tests, sph_tests, terminated;
    int64_t samples_skipped;
    double  start_ms;      /* start of the launch after the frame's first launch
                              (launches on the side stream overlap the others) */
} gxy_generation_stats;
int gxy_gpu_set_profiling(gxy_scene scene, int on);

/* Process-wide tuning knobs chosen by galaxy_gb300.autotune:
 * GXY_TUNE_BLOCKS_PER_SM: 2 (128 registers per thread) or 3 (80 registers)
 *   -- the register budget the wavefront kernels are compiled for;
 * GXY_TUNE_GRID_PER_SM: blocks per SM of the grid-stride frame kernels;
 * GXY_TUNE_SPLIT_SECONDARY: see below. */
#define GXY_TUNE_BLOCKS_PER_SM 1
#define GXY_TUNE_GRID_PER_SM   2
#define GXY_TUNE_SPLIT_SECONDARY 3   /* 1: shadow/AO rays of volume scenes traced as a query
                                        pass plus a march pass with per-lane refill */
#define GXY_TUNE_SPLIT_PRIMARY   4   /* 1: camera rays of volume scenes likewise */
#define GXY_TUNE_BVH_SAH         5   /* top of the BVH binary tree rebuilt by binned SAH
                                        over radix-tree clusters of at most C primitives:
                                        0 off (radix tree only), 1 C = 256, >= 2 C itself.
                                        Applies to scenes committed afterwards */
#define GXY_TUNE_LEAF_MAX        6   /* largest primitive count of a BVH8 leaf, 1-4
                                        (default 1); scenes committed afterwards */
#define GXY_TUNE_TRAV_STEPS      7   /* BVH8 node visits per refill round of the query
                                        passes, 1-64 (default 8) */
#define GXY_TUNE_MARCH_STEPS     8   /* volume samples per refill round of the march
                                        passes, 1-256 (default 16) */
#define GXY_TUNE_CAMERA_PACKET   9   /* 1 (default): camera rays of a frame, and of a batch of
                                        jobs of one volume scene, queried by warps over 8x4
                                        pixel tiles (a batch's tiles job by job) with one shared
                                        BVH8 traversal; 0: per-lane refill traversal */
#define GXY_TUNE_SKIP_CLEAR     10   /* read at scene commit.  1 (default): flag the volume
                                        bricks whose samples all lie below the transfer
                                        function's zero-opacity threshold; the march
                                        passes then read no voxels for intervals between
                                        two such positions (same images and counters);
                                        0: no flags, every sample read */
#define GXY_TUNE_SKIP_MODE      11   /* clear-brick skipping per pass, bits (default 9):
                                        1: the camera-ray march also advances
                                        through the rest of a flagged brick in one run of
                                        distance updates (it always skips per position
                                        and jumps runs of clear 32^3 superbricks);
                                        2: the shadow/AO march jumps runs of clear
                                        superbricks at its first position and after each
                                        refill round, sampling every other position;
                                        4: the shadow/AO march skips as the camera-ray
                                        march does (incoherent rays: a warp runs both
                                        paths when its lanes differ);
                                        8 (default): occlusion shortcut -- a shadow/AO ray whose
                                        march positions in its partition all lie in clear
                                        superbricks ends at the first surface the query
                                        finds before the partition exit, unmarched (same
                                        frames; fewer samples, node visits and primitive
                                        tests counted) */
#define GXY_TUNE_QUEUE_LIMIT    14   /* largest ray-queue buffer of the frame path, in records
                                        (0, default: none but the HBM budget).  Queues grow to
                                        the worst case of the next launch; a frame whose camera
                                        rays do not fit is rendered in bands of image rows; a
                                        later generation that still runs out of room reports
                                        GXY_ERR_OVERFLOW */
#define GXY_TUNE_RUNAHEAD       19   /* frame path: most generations launched per host read of
                                        the queue counts, 1-16 (default 16).  After the camera
                                        generation the host reads the three counts once per
                                        block; a block runs to the generation count of the
                                        scene's previous frame, and its later generations take
                                        their input counts from device memory.  Its queues are
                                        grown to the worst case of the whole block beforehand;
                                        the block is shortened where the queue set still being
                                        read holds too little room.  A scene's first frame, and
                                        a frame that outlasts the previous one, read after every
                                        generation; 1: always so */
#define GXY_TUNE_BVH_COLLAPSE   18   /* read at scene commit.  How binary BVH nodes are grouped
                                        into 8-wide nodes: 1 (default) the grouping of least summed
                                        wide-node surface area, by a dynamic programme over the
                                        tree (single-primitive leaves, no SAH top); 0 the greedy
                                        rule, opening the child of largest area first */
#define GXY_TUNE_SEC_PACKET     17   /* shadow/AO query of a frame: 0 (default) one lane per ray
                                        with refill; 1 one warp per 32 consecutive rays with a
                                        shared BVH8 traversal (same frames) */
#define GXY_TUNE_SPLIT_HANDOFF  16   /* 1 (default): primaries handed to the next partition of a
                                        volume scene are traced as camera rays are, a query pass
                                        plus the camera-ray march with clear-brick skipping; 0: one
                                        pass per ray (same frames) */
#define GXY_TUNE_QUEUE_CHUNK    15   /* shadow/AO query: records per 256-thread block taken from
                                        the ray queue at once, 256-65536; each of the block's 8
                                        warps takes 1/8 of them as one consecutive run and hands
                                        them to its idle lanes in queue order (0, default: a warp
                                        takes exactly what its idle lanes need) */
#define GXY_TUNE_QUERY_BLOCKS   20   /* with GXY_TUNE_BLOCKS_PER_SM 3: resident blocks per SM of the
                                        shadow/AO query, 2 (128 registers per thread), 3 (default:
                                        80 registers) or 4 (64 registers); the other refill
                                        queries run at 4 */
#define GXY_TUNE_PMARCH_BLOCKS  21   /* with GXY_TUNE_BLOCKS_PER_SM 3: resident blocks per SM of the
                                        camera-ray march (and of handed-off primaries), 2 (default:
                                        128 registers per thread) or 3 (80 registers) */
#define GXY_TUNE_PQUERY_BLOCKS  22   /* with GXY_TUNE_BLOCKS_PER_SM 3: resident blocks per SM of a
                                        frame's warp-cooperative camera query and handed-off primary
                                        query and of a batch's camera query, 2 (default: 128
                                        registers per thread) or 4 (64) */
#define GXY_TUNE_CONTINUE       23   /* 1 (default): in a frame, a shadow/AO ray that moves to the
                                        next brick, carrying its query's closest hit
                                        (GXY_TUNE_CARRY_HITS), is set up for that brick and marches
                                        on in the same lane instead of waiting for the next
                                        generation; 0: hand it on through the queues (same frames) */
#define GXY_TUNE_CARRY_HITS     13   /* 1 (default): a shadow/AO ray that moves to the next
                                        partition carries the closest hit its query found
                                        over its whole extent, and the next partition's
                                        query reuses it instead of traversing again (the
                                        same hit, except for a surface within float
                                        rounding of the shared face); 0: query again */
/* The threshold the empty-space skipping uses (no counterpart in the
 * reference): the largest T such that every data value below T, and NaN,
 * has opacity exactly 0 in the transfer-function lookup; -inf when the
 * lowest entry's opacity is positive, +inf when every entry's is zero.
 * Host only: needs neither a device nor gxy_gpu_init. */
int gxy_tf_clear_below(const gxy_tf *tf, float *threshold);
int gxy_gpu_set_tuning(int knob, int value);
int gxy_gpu_get_tuning(int knob, int *value);
int gxy_gpu_query_generations(gxy_scene scene, gxy_generation_stats *out, int max, int32_t *n);

/* ---- batched frames (many Renderings in one launch) --------------------
 *
 * Replaces RenderingSet's per-Rendering processing (RenderingSet.cpp:700-738)
 * and gxywriter's camera x visualization loop (gxywriter.cpp:181-219) with
 * one persistent, cooperative wavefront launch per batch: every job's camera
 * rays and every later generation of shadow, AO and handed-off rays of all
 * jobs share the device queues, with a grid barrier between generations and
 * no host round trip.  A batch slot owns its queues, job table and stream;
 * several slots run concurrently (continuous batching in the serving loop). */
typedef struct gxy_job {
    gxy_scene    scene;
    gxy_camera   camera;
    gxy_lighting lighting;   /* resolved (no camera-relative lights) */
    float       *fb_rgba;    /* device framebuffer, width*height*4 fp32; contributions added */
} gxy_job;

typedef struct gxy_batch_s *gxy_batch;
/* Queue memory for max_pixels camera rays per submission with up to
 * max_shadow (lights) and max_ao secondary rays per pixel; GXY_ERR_ADMISSION
 * if it does not fit the HBM budget. */
int gxy_gpu_batch_create(int64_t max_pixels, int max_jobs, int max_shadow, int max_ao, gxy_batch *out);
int gxy_gpu_batch_release(gxy_batch batch);
/* Asynchronous submission on the batch's own stream.  flags:
 * GXY_BATCH_GRAPH replays the submission (job-table upload, counter reset,
 * launches, status read-back) as a CUDA graph updated in place between
 * submissions; GXY_BATCH_COOPERATIVE runs all generations in one cooperative
 * launch with grid barriers (lowest launch overhead, but the launch holds the
 * whole GPU), otherwise each generation is its own launch reading the
 * previous generation's queue counts from device memory (up to 10
 * generations), so batches on different streams overlap. */
#define GXY_BATCH_GRAPH        1
#define GXY_BATCH_COOPERATIVE  2
int gxy_gpu_batch_submit(gxy_batch batch, const gxy_job *jobs, int n_jobs, int flags);
/* *done = 1 once the last submission finished (its status is then checked). */
int gxy_gpu_batch_poll(gxy_batch batch, int *done);
/* Bounded host wait for the last submission (GXY_ERR_TIMEOUT after timeout_ms). */
int gxy_gpu_batch_wait(gxy_batch batch, int timeout_ms);
int gxy_gpu_batch_counters(gxy_batch batch, gxy_counters *out);
/* The cudaStream_t of the batch (for events and framebuffer copies). */
int gxy_gpu_batch_stream(gxy_batch batch, void **stream);

/* ---- Serving loop -------------------------------------------------------
 * Replaces the request handling of Galaxy's serving front ends
 * (ViewerClientServer::handle `render`, src/multiserver/ViewerClientServer.cpp:
 * 62-253; GuiClientServer gui::render, src/guiserver/GuiClientServer.cpp:375-407),
 * which render one request at a time, with continuous batching: a worker
 * thread admits submitted requests into n_slots batch slots as slots and the
 * framebuffer budget allow (requests up to small_pixels of one scene packed
 * up to small_batch_pixels per launch, larger ones alone; a large request
 * lets smaller ones pass for at most big_wait_s), and finds completions by
 * polling.  Framebuffers come from a stream-ordered device memory pool. */
typedef struct gxy_server_s *gxy_server;
typedef struct gxy_server_config {
    int32_t n_slots;
    int64_t slot_pixels;          /* camera rays per slot = largest request */
    int32_t max_jobs, max_shadow, max_ao;
    size_t  fb_budget_bytes;      /* device framebuffers of admitted requests */
    int64_t small_pixels;
    int64_t small_batch_pixels;
    double  big_wait_s;
    int32_t use_graph;            /* GXY_BATCH_GRAPH submissions */
    int32_t cooperative;          /* GXY_BATCH_COOPERATIVE submissions */
} gxy_server_config;
int gxy_server_create(const gxy_server_config *config, gxy_server *out);
/* Waits (bounded) for running batches, then frees everything. */
int gxy_server_release(gxy_server server);
/* Enqueue a request arriving now (lighting resolved); GXY_ERR_ADMISSION if
 * it can never be admitted (larger than a slot or the framebuffer budget). */
int gxy_server_submit(gxy_server server, gxy_scene scene, const gxy_camera *camera,
                      const gxy_lighting *lighting, int64_t *id);
int gxy_server_poll(gxy_server server, int64_t id, int *done);
/* Cancel a request (no counterpart in Galaxy, whose servers render each
 * request to the end): a waiting request is removed at once; a running one
 * finishes its batch (the other requests in it are unaffected) and its image
 * is discarded.  gxy_server_take then returns GXY_ERR_CANCELLED for it.
 * *was_running (may be NULL) tells which case applied. */
int gxy_server_cancel(gxy_server server, int64_t id, int *was_running);
/* Bounded host wait until every submitted request has finished. */
int gxy_server_drain(gxy_server server, int timeout_ms);
/* Copy a finished request's image to host rgba (height*width*4 fp32, or
 * NULL) and release it; latency_s = submission to completion, rays = its
 * share of the batch's traced rays. */
int gxy_server_take(gxy_server server, int64_t id, float *rgba, double *latency_s, int64_t *rays);

/* ---- RayList-level drop-in (host buffers) ------------------------------ */

/* Camera::generate_initial_rays for partition `partition`: fills `out`
 * (capacity out->n on entry) and sets *n_out to the rays emitted. */
int gxy_gpu_generate_initial_rays(gxy_scene scene, int partition, const gxy_camera *camera,
                                  gxy_raylist *out, int32_t *n_out);
/* TraceRays::Trace for the rays of `in` inside partition `partition`:
 * updates `in` in place and writes the secondary list (AO block first, then
 * shadow block, as TraceRays.cpp:89-117 orders it) into `out` (capacity
 * out->n on entry); *n_out receives its length. */
int gxy_gpu_trace_raylist(gxy_scene scene, int partition, const gxy_lighting *lighting,
                          gxy_raylist *in, gxy_raylist *out, int32_t *n_out);
int gxy_gpu_classify(gxy_raylist *rays);
int gxy_gpu_assign_destinations(gxy_scene scene, int partition, gxy_raylist *rays);
/* Adds every TERMINATED ray's (r,g,b,o) to host framebuffer fb (w*h*4). */
int gxy_gpu_accumulate_terminated(const gxy_raylist *rays, float *fb_rgba, int width, int height);

/* ---- Allocation-free camera rays ----------------------------------------
 * No counterpart in the reference.  gxy_gpu_generate_initial_rays with no
 * device allocation, for callers that must not call cudaMalloc or cudaFree:
 * e.g. a visualization step run in situ inside a simulation whose own
 * allocator holds the GPU's memory, where a cudaFree would synchronise the
 * whole device and stall the simulation's streams.  The caller passes the
 * output RayList in memory the GPU can address (device memory of the current
 * device, managed memory, or mapped pinned host memory); each of the 25
 * arrays must hold out->n records -- the whole range is checked before
 * anything is written (for device and managed memory it must lie inside one
 * allocation), and a shorter or unaddressable array is refused with
 * GXY_ERR_INVALID.  The result equals gxy_gpu_generate_initial_rays's.
 * Scratch is a fixed 8.25 MiB array in this library's device image, held on
 * every GPU that loads the library until the process exits.  Images above
 * 1048576 pixels (1024 x 1024) are refused with GXY_ERR_INVALID.
 * The first call on each device looks up the array's device address (with
 * that device current).  Under CUDA's default lazy module loading that first
 * call also loads the library's device code there, and with it the 8.25 MiB
 * array: make the first call (or set CUDA_MODULE_LOADING=EAGER) before the
 * simulation's allocator reserves the device memory, and before any stream
 * capture.  Later calls re-check the cached address and look it up again
 * after a cudaDeviceReset.  All calls on a device share the array, so calls
 * that overlap on the GPU (from several host threads) race: serialise them.
 * The work runs on the calling thread's per-thread default stream
 * (cudaStreamPerThread), so it waits for no other stream except the legacy
 * default stream, and the call returns after the rays are written. */
int gxy_gpu_generate_initial_rays_noalloc(gxy_scene scene, int partition, const gxy_camera *camera,
                                          gxy_raylist *out, int32_t *n_out);

#ifdef __cplusplus
}
#endif
#endif /* GXY_GPU_H */
