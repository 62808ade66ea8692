/*
 * pms.h -- C ABI of libpms, the GB300-native particle-to-surface pipeline.
 *
 * libpms reimplements, for one GB300 (sm_103a), the per-frame hot path of the
 * reference VisFluid program (xiaoxiaoyu1872/PostMPS): spatial hashing,
 * surface-particle detection, anisotropic kernels, narrow-band vertex
 * detection, narrow-band scalar field, marching cubes and diffuse-particle
 * generation.  The reference exposes that path only as a C++ class chain
 * (GPUPOST -> NeighborSearch / SurfaceReconstruction(Anisotropic,
 * MarchingCube) / DiffuseGeneration sharing one GPUmemory); every entry point
 * below names the member function it replaces.
 *
 * Conventions
 *   - Every call returns pms_status; PMS_OK == 0.  A failing call leaves a
 *     message retrievable with pms_last_error(ctx).  Nothing aborts.
 *   - Host buffers are caller-owned plain arrays; positions and velocities are
 *     xyz-interleaved float32 (the reference's float3 layout).
 *   - Device buffers are owned by the context and reused (grow-only) across
 *     frames.  A context is bound to one device and one CUDA stream (its copy
 *     and staging streams run beside it and are waited for explicitly; the
 *     diffuse stream of pms_run_frame is forked from it and joined back within
 *     the call) and is not thread-safe; use one context per host thread
 *     (pms_stage_particles is the one call another thread may make).
 *   - Counts stay on the device between stages; calls that return counts or
 *     data synchronise the context's stream.
 */
#ifndef PMS_H
#define PMS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PMS_ABI_VERSION 1

typedef enum pms_status {
    PMS_OK = 0,
    PMS_ERR_INVALID_ARGUMENT = 1,  /* null pointer, bad size, bad enum */
    PMS_ERR_CUDA = 2,              /* a CUDA runtime call failed */
    PMS_ERR_OUT_OF_MEMORY = 3,     /* device or host allocation failed */
    PMS_ERR_CAPACITY = 4,          /* a caller-provided buffer or a fixed cap is too small */
    PMS_ERR_IO = 5,                /* file could not be read or written */
    PMS_ERR_CONFIG = 6,            /* config.txt missing or unusable */
    PMS_ERR_STATE = 7,             /* stage called before its inputs exist */
    PMS_ERR_TIMEOUT = 8,           /* a bounded device wait gave up */
    PMS_ERR_UNSUPPORTED = 9        /* input outside what the kernels handle */
} pms_status;

/* ---------------------------------------------------------------------------
 * Configuration: the reference's config.txt (Params.cpp:24-152, Define.h:85-202)
 * ------------------------------------------------------------------------- */
typedef struct pms_config {
    /* [Sim] */
    double mass;                       /* Mass (default 0) */
    double particle_spacing;           /* ParticleSpacing (0.01) */
    /* [Surface] */
    double smoothing_radius_ratio;     /* SmoothingRadiusRatio (4), truncated to int */
    long   min_num_neighbors;          /* MinNumNeighbors (8) */
    long   isolate_num_neighbors;      /* IsolateNumNeighbors (4) */
    double lambda_for_smoothed;        /* LambdaForSmoothed (0.5) */
    double iso_value;                  /* IsoValue (0.5) */
    /* [Diffuse] */
    double min_wave_crests, max_wave_crests;        /* Min/MaxWaveCrestsThreshold (0, 100) */
    double min_trapped_air, max_trapped_air;        /* Min/MaxTrappedAirThreshold (0, 100) */
    double min_kinetic_energy, max_kinetic_energy;  /* Min/MaxKineticEnergyThreshold (0, 100) */
    double trapped_air_multiplier;     /* DiffuseTrappedAirMultiplier (800) */
    double wave_crests_multiplier;     /* DiffuseWaveCrestsMultiplier (4000) */
    double time_step;                  /* TimeStep (0.01) */
    double life_time;                  /* LifefimeMultiplier (10) */
    double buoyancy_control;           /* BuoyancyControl (0.8) */
    double drag_control;               /* DragControl (0.5) */
    /* [Domain] */
    double sp_scale;                   /* SpatialGridSizeScale (2) */
    double sc_scale;                   /* SclarGridSizeScale (2) */
    double domain_min[3], domain_max[3]; /* Min_x.. / Max_x.. (unused: the grid follows each frame's bbox) */
    /* [Config] */
    int gpu_id;                        /* GpuId (0) */
    int frame_start, frame_end, frame_step;  /* Framefrom (0), Frameto (10), FrameStep (1) */
    int num_zeros;                     /* NumZeros (4) */
    int is_surface;                    /* IsSurfaceReconstruct (false) */
    int is_diffuse;                    /* IsDiffuseGeneration (true) */
    char fluid_path[512], fluid_prefix[128];
    char surface_path[512], surface_prefix[128];
    char diffuse_path[512], diffuse_prefix[128];
    /* GB300 build additions (no reference counterpart) */
    double fp64_svd_cond;              /* covariances with condition number above this use the FP64 eigen solver (1e6) */
    uint64_t rng_seed;                 /* seed of the diffuse spawn uniforms (replaces std::random_device) */
    char band_model[512];              /* [GB300] BandModel: learned-band model file; empty = plain band */
    int ply_binary;                    /* [GB300] PlyBinary: pms_run_config writes binary PLY (false: ASCII) */
    int weld_mesh;                     /* [GB300] WeldMesh: ... an indexed mesh (false: the reference's soup) */
} pms_config;

/* Derived float32 parameters (SimParams, SurfaceParams, DiffuseParams, Define.h:85-139). */
typedef struct pms_params {
    float mass, particle_spacing;
    int   smoothing_radius_ratio;
    float h, h_inv, h_sq, aniso_radius;
    int   min_num_neighbors, isolate_num_neighbors;
    float lambda_for_smoothed, iso_value;
    float hd, hd_inv, hd_sq, hd_aniso, coefficient;
    int   d_min_num_neighbors;
    float min_wc, max_wc, min_ta, max_ta, min_ke, max_ke;
    int   ta_mult, wc_mult, life_time;
    float time_step, buoyancy, drag;
    int   sp_scale, sc_scale;
    float sp_grid_size, sc_grid_size;
    int   spexpand, scexpand, spexpand_diffuse;
} pms_params;

/* Per-frame grid (GridParams, Define.h:142-174). */
typedef struct pms_grid {
    float min_pos[3], max_pos[3];      /* spatial grid: bbox -/+ 4h */
    float scmin_pos[3], scmax_pos[3];  /* scalar grid: bbox -/+ 2h */
    float sp_grid_size, sc_grid_size;
    uint32_t spres[3], scres[3];
    int32_t spexpand, scexpand, spexpand_diffuse;
    uint32_t sp_size, sc_size;
} pms_grid;

/* Counters of one frame (GPUmemory.h:17-31). */
typedef struct pms_counts {
    uint32_t n_particles;
    uint32_t n_surface_particles;      /* NumSurfaceParticles */
    uint32_t n_band_vertices;          /* NumSurfaceVertices */
    uint32_t n_valid_cubes;            /* NumValidSurfaceCubes */
    uint64_t n_mesh_vertices;          /* NumSurfaceMeshVertices (3 per triangle) */
    uint32_t n_free_surface;           /* NumFreeSurfaceParticles */
    uint32_t n_generated_diffuse;      /* GeneratedNumDiffuseParticles */
    uint32_t n_spawning;               /* NumIsDiffuseParticles */
    uint32_t n_diffuse;                /* OldNumDiffuseParticles after delete/append */
    uint32_t n_spray, n_foam, n_bubble;
    uint32_t n_fp64_svd;               /* covariances re-solved in FP64 */
    /* learned / certified band (pms_band_learned); zero after the plain band */
    uint32_t n_band_candidates;        /* cubes the network evaluated */
    uint32_t n_band_predicted;         /* cubes it predicted crossed */
    uint32_t n_band_exact;             /* band vertices evaluated exactly first (corners of predicted cubes) */
    uint32_t n_band_certified;         /* band vertices certified above iso without an exact value */
    uint32_t n_band_rechecked;         /* ... of those, corners of valid cubes, then evaluated exactly */
    uint64_t n_field_pairs;            /* (band vertex, particle) pairs the field evaluated this frame */
} pms_counts;

typedef struct pms_ctx pms_ctx;

/* Parses config.txt with the reference's INI rules (inih: case-insensitive
 * keys, ';' inline and '#'/';' line comments, continuation lines) and its
 * defaults.  Replaces Params::setFilname/setParams (Params.cpp:17-152). */
pms_status pms_config_default(pms_config* out);
pms_status pms_config_load(const char* path, pms_config* out);

/* Bit-exact restatement of Params.cpp:53-118. */
pms_status pms_params_derive(const pms_config* cfg, pms_params* out);

/* Bit-exact restatement of the per-frame grid, FileData.cpp:259-279 (NOBOUND). */
pms_status pms_grid_from_bbox(const pms_params* p, const float bmin[3], const float bmax[3], pms_grid* out);

/* Context lifetime: GPUPOST::initialize (GPUPOST.cpp:20-31) and
 * GPUmemory::initGPUmemory (GPUmemory.cpp:14-18).  device < 0 uses cfg->gpu_id. */
pms_status pms_create(const pms_config* cfg, int device, pms_ctx** out);
void       pms_destroy(pms_ctx* ctx);
const char* pms_last_error(const pms_ctx* ctx);
const char* pms_status_string(pms_status s);

/* Runs the context on a caller-provided cudaStream_t (NULL: the context's own stream). */
pms_status pms_set_stream(pms_ctx* ctx, void* cuda_stream);

/* Preallocates device buffers for frames up to these sizes (0: leave as is).
 * GPUmemory's per-frame cudaMalloc/cudaFree pairs (GPUmemory.cpp:47-363) are
 * replaced by this grow-only reservation. */
pms_status pms_reserve(pms_ctx* ctx, uint32_t max_particles, uint64_t max_scalar_vertices);

/* Uploads one frame from host arrays (vel may be NULL -> zeros).  rhop may be
 * NULL and is not read: every stage uses the density recomputed from the
 * positions, as the reference overwrites Rhop before its first use
 * (Anisotropic_kernel.cuh:212).  Replaces FileData::loadFluidFile +
 * GPUmemory::memAlcandCpy_fluid (FileData.cpp:214-305, GPUmemory.cpp:47-72). */
pms_status pms_upload_particles(pms_ctx* ctx, const float* pos_xyz, const float* vel_xyz,
                                const float* rhop, uint32_t n);
/* Same, from device-resident arrays (copied device-to-device on the context stream). */
pms_status pms_upload_particles_device(pms_ctx* ctx, const float* d_pos_xyz, const float* d_vel_xyz,
                                       const float* d_rhop, uint32_t n);

/* Staged upload (no counterpart in the reference, whose loadFluidFile reads and
 * copies each frame after the last one finished, FileData.cpp:177-305).
 * pms_stage_particles copies the next frame's host arrays into pinned staging
 * (split over the host's threads) and from there, on a stream of its own, into a
 * second pair of device input buffers; it may run on another host thread while
 * pms_run_frame runs the current frame on this context, so the parse and the
 * host-to-device copy of frame k + 1 overlap frame k.  pms_upload_staged then
 * makes the staged frame the context's input (a buffer swap and a device-side
 * wait, no copy), in place of pms_upload_particles.  One frame is staged at a
 * time (PMS_ERR_STATE while one waits); stage the next one only after
 * pms_upload_staged of the last returned.  Staging reports errors by status
 * only; pms_last_error belongs to the thread running the frames. */
pms_status pms_stage_particles(pms_ctx* ctx, const float* pos_xyz, const float* vel_xyz, const float* rhop, uint32_t n);
pms_status pms_upload_staged(pms_ctx* ctx);

/* Stages (asynchronous on the context stream unless stated). */
pms_status pms_build_grid(pms_ctx* ctx);        /* NeighborSearch::SpatialGridBuilding, NeighborSearch.cu:37-76 */
pms_status pms_anisotropy(pms_ctx* ctx);        /* Anisotropic::processingOfParticles, Anisotropic.cu:30-40 */
pms_status pms_band(pms_ctx* ctx);              /* Anisotropic::processingOfVertices, Anisotropic.cu:43-50 */
pms_status pms_field(pms_ctx* ctx);             /* Anisotropic::estimationOfscalarField, Anisotropic.cu:53-56 */
pms_status pms_marching_cubes(pms_ctx* ctx);    /* MarchingCube::triangulation, MarchingCube.cu:32-68 */
pms_status pms_surface(pms_ctx* ctx);           /* SurfaceReconstruction::runsimulation, SurfaceReconstruction.cu:34-60 */
pms_status pms_diffuse(pms_ctx* ctx);           /* DiffuseGeneration::runsimulation, DiffuseGeneration.cu:89-104 */
/* One iteration of GPUPOST::runSimulation (GPUPOST.cpp:56-81): grid, then surface and
 * diffuse as configured.  With both on, the diffuse stage runs on a stream of the
 * context's own beside the band, field and marching cubes, forked after the
 * anisotropy pass and joined back into the context's stream before the call returns;
 * results are those of the stages one after the other. */
pms_status pms_run_frame(pms_ctx* ctx);

/* Density and velocity at every mesh vertex: MarchingCube::scalarvalue /
 * estimationOfScalarValue (MarchingCube.cu:153-163, MarchingCube_kernel.cuh:161-233),
 * which the reference runs after the triangles; here on request (the reference
 * only writes them from FileData::saveSurfaceVTKfile, which its frame loop does
 * not call).  After pms_marching_cubes. */
pms_status pms_scalar_values(pms_ctx* ctx);

/* Results (synchronise the stream). */
pms_status pms_get_counts(pms_ctx* ctx, pms_counts* out);
pms_status pms_get_grid(pms_ctx* ctx, pms_grid* out);
/* Triangle soup, 3 vertices per triangle (positions and normals xyz float32);
 * nrm_xyz may be NULL.  Replaces the D2H copies of FileData::saveSurfacePLYfile
 * (FileData.cpp:1297-1300).  *n_vertices receives the count even on PMS_ERR_CAPACITY.
 * The marching cubes make the normals only when a streamed mesh asked for them;
 * otherwise the first call that passes nrm_xyz makes them (one more emission pass). */
pms_status pms_download_mesh(pms_ctx* ctx, float* pos_xyz, float* nrm_xyz, uint64_t cap_vertices,
                             uint64_t* n_vertices);
/* Registers host buffers (page-locked, e.g. cudaHostAlloc or cudaHostRegister,
 * for the copy to overlap) that every following pms_marching_cubes fills with
 * the frame's triangle soup on a copy stream of its own, while the stages after
 * it (diffuse generation) run; nrm_xyz may be NULL, pos_xyz NULL unregisters.
 * pms_wait_mesh blocks until the copy has landed and returns the vertex count
 * (PMS_ERR_CAPACITY, with the count, when cap_vertices was too small; nothing
 * is copied then).  The emission runs in vertex ranges and each range is copied
 * while the next is made (one range when an earlier frame's copy is still in
 * flight: the copy then overlaps the next frame anyway).
 * Frames in flight: each frame's copy keeps the buffers registered when it ran,
 * and registering others does not wait for it.  pms_wait_mesh waits for the
 * oldest frame not yet waited for.  So a caller that alternates two buffer sets
 * can run frame k+1 before waiting for frame k, whose copy then overlaps frame
 * k+1's stages.  A frame that streams into buffers that an earlier frame's
 * pending copy also writes drops that earlier frame (and every older pending
 * one) after its copy has landed, as does a fifth frame in flight for the
 * oldest.  With one buffer set this is the plain case: each frame replaces the
 * last, and the wait returns the newest.  Buffers stay valid until their frame's
 * wait.  No counterpart in the reference, which copies the soup back with a
 * blocking cudaMemcpy when it writes the PLY file (FileData.cpp:1300-1305). */
pms_status pms_stream_mesh_to_host(pms_ctx* ctx, float* pos_xyz, float* nrm_xyz, uint64_t cap_vertices);
pms_status pms_wait_mesh(pms_ctx* ctx, uint64_t* n_vertices);
/* Welded (indexed) mesh of the current frame, after pms_marching_cubes: one vertex
 * per crossed grid edge and a triangle index list in the soup's triangle order
 * (3 indices per triangle, n_indices = the soup's vertex count).  Each edge point is
 * interpolated once, from the edge's lower to its upper corner; the soup interpolates
 * it in every cube that uses it from the end that cube's table names first, so the
 * two agree up to that rounding.  With normals != 0 the vertex normals are made too
 * (as the soup's, from central differences of the field).  No counterpart in the
 * reference, whose PLY and VTK surface files hold the triangle soup
 * (FileData.cpp:677-773, 1277-1332); a welded mesh is about 2.4x smaller. */
pms_status pms_weld_mesh(pms_ctx* ctx, int normals);
pms_status pms_download_welded_mesh(pms_ctx* ctx, float* pos_xyz, float* nrm_xyz, uint64_t cap_vertices,
                                    uint32_t* indices, uint64_t cap_indices, uint64_t* n_vertices, uint64_t* n_indices);
/* The scalar values of the mesh vertices (any array may be NULL): velocity xyz,
 * its length and the density (the reference's ScalarValue). */
pms_status pms_download_scalar_values(pms_ctx* ctx, float* vel_xyz, float* vel_len, float* rhop, uint64_t cap,
                                      uint64_t* n_vertices);
/* Live diffuse particles of one type (0 spray, 1 foam, 2 bubble, -1 all), in the
 * reference's generated-then-old order (DiffuseGeneration.cu:760-867).  Any of
 * the arrays may be NULL; ttl is int32, energies are float32. */
pms_status pms_download_diffuse(pms_ctx* ctx, int type, float* pos_xyz, float* vel_xyz, int32_t* type_out,
                                int32_t* ttl, float* wave_crest, float* trapped_air, float* energy,
                                uint32_t cap, uint32_t* n_out);

/* One live diffuse particle as the library keeps it (32 bytes). */
typedef struct pms_diffuse_particle {
    float pos[3];
    int32_t ttl;
    float vel[3];
    int32_t type;                      /* 0 spray, 1 foam, 2 bubble (the reference's classes) */
} pms_diffuse_particle;
/* Registers a host buffer (page-locked for the copy to overlap) that every
 * following pms_diffuse fills with the frame's live diffuse particles, in the
 * order of pms_download_diffuse, with one copy on the context's copy stream; out
 * NULL unregisters.  pms_wait_diffuse blocks until it has landed and returns the
 * count (PMS_ERR_CAPACITY, with the count, when cap was too small; nothing is
 * copied then).  The next frame's diffuse stage waits on the device for the copy
 * before it moves those particles.  Frames in flight, their buffers and the
 * order of the waits work as for pms_stream_mesh_to_host, with a queue of their
 * own.  No counterpart in the reference, which copies
 * the particles back with blocking cudaMemcpy calls to write its diffuse files
 * (DiffuseGeneration.cu:760-867). */
pms_status pms_stream_diffuse_to_host(pms_ctx* ctx, pms_diffuse_particle* out, uint64_t cap);
pms_status pms_wait_diffuse(pms_ctx* ctx, uint64_t* n);

/* Drops the diffuse particles carried between frames and restarts the frame
 * counter that seeds the spawn, so the next frame starts a sequence as a fresh
 * run does (the reference's DiffuseGeneration starts empty and has no reset;
 * DiffuseGeneration.cu:21-87).  Waits for the streamed copies still in flight;
 * their frames can still be waited for with pms_wait_diffuse. */
pms_status pms_reset_diffuse(pms_ctx* ctx);

/* Intermediate arrays, for parity tests.  Bytes needed are written to *needed;
 * nothing is copied when dst is NULL or cap_bytes is too small. */
typedef enum pms_array {
    PMS_ARRAY_KEYS_SORTED = 1,   /* uint32[n]  cell key of each sorted particle */
    PMS_ARRAY_PERM = 2,          /* uint32[n]  input index of each sorted particle */
    PMS_ARRAY_CELL_START = 3,    /* uint32[sp_size]  (0 for empty cells, as the reference) */
    PMS_ARRAY_CELL_END = 4,      /* uint32[sp_size] */
    PMS_ARRAY_SURF_COUNT = 5,    /* uint32[sp_size]  numSurParticleGrid */
    PMS_ARRAY_SURF_LIST = 6,     /* uint32[ns]  sorted index of each surface particle */
    PMS_ARRAY_DENSITY = 7,       /* float[n]   density of each sorted particle */
    PMS_ARRAY_MEAN = 8,          /* float[3 ns] weighted mean of each surface particle */
    PMS_ARRAY_G = 9,             /* float[10 ns] G row-major + maxvalue (MatrixValue layout) */
    PMS_ARRAY_NORMAL = 10,       /* float[3 ns] oriented normal of each surface particle */
    PMS_ARRAY_FLAG = 11,         /* uint8[ns]  thin-feature / isolated flag */
    PMS_ARRAY_BAND_BITMAP = 12,  /* uint32[ceil(sc_size/32)] band-vertex bitmap */
    PMS_ARRAY_BAND_LIST = 13,    /* uint32[nv] band vertices, ascending linear index */
    PMS_ARRAY_FIELD = 14,        /* float[nv] scalar field at band vertices */
    PMS_ARRAY_CUBE_CASE = 15,    /* uint32[nv] marching-cubes case (0 when not all corners are band) */
    PMS_ARRAY_CUBE_NVERT = 16,   /* uint32[nv] mesh vertices emitted by each cube */
    PMS_ARRAY_POS_SORTED = 17,   /* float[3 n] sorted positions */
    PMS_ARRAY_NEIGHBORS = 18,    /* uint32[ns] neighbours within h of each surface particle */
    PMS_ARRAY_DIFFUSE_POTENTIAL = 19, /* float[3 n] waveCrest, Ita, energy after the phi clamps */
    PMS_ARRAY_DIFFUSE_COUNT = 20,     /* int32[n] spawned diffuse particles per sorted particle */
    PMS_ARRAY_FREE_NORMAL = 21,       /* float[3 n] particle normals after the diffuse colour-gradient pass */
    PMS_ARRAY_BAND_CERTIFIED = 22     /* uint32 bitmap over the scalar grid: band vertices of a learned or
                                         certified band whose field value is a placeholder above iso */
} pms_array;
pms_status pms_debug_download(pms_ctx* ctx, int array_id, void* dst, uint64_t cap_bytes, uint64_t* needed);
/* Tests of the failure path: the first bounded wait of the band network on the
 * tensor cores gives up after `polls` polls (0: at once; negative: the default
 * bound).  A wait that gives up sets an error the next pms_get_counts reports
 * ("a wait on the tensor cores timed out"); a second bounded wait lets the
 * work in flight finish before the kernel frees its tensor memory, so the
 * context stays usable.  No reference counterpart. */
pms_status pms_debug_set_wait_limit(pms_ctx* ctx, int64_t polls);

/* Device time of each stage of the last frame, in milliseconds (CUDA events on
 * the context stream): [grid, anisotropy, band, field, marching cubes, diffuse].
 * When pms_run_frame ran the diffuse stage beside the surface stages, its figure
 * is the span from the anisotropy's end to its own end. */
pms_status pms_stage_times(pms_ctx* ctx, float* ms, int count);

/* Number of kernels libpms launched since the context was created. */
uint64_t pms_kernel_launches(const pms_ctx* ctx);

/* Copies the marching-cubes tables in use (derived != 0: the tables libpms
 * derives itself when built without the reference tree).  Returns 1 when the
 * active tables are the reference's (MarchingCubesHelper.cpp:3-587), else 0. */
int pms_mc_tables(uint32_t* edge_flags /*256*/, int32_t* tri /*256*16*/, uint32_t* num_vertices /*256*/,
                  uint32_t* edge_vertices /*24*/, int derived);

/* ---------------------------------------------------------------------------
 * Learned narrow band.  No counterpart in the reference: it reshapes how the
 * field (Anisotropic_kernel.cuh:656-777) is evaluated over the reference's own
 * band (estimationOfSurfaceVertices, Anisotropic_kernel.cuh:522-636).  A
 * 64 -> 64 -> 1 ReLU MLP with BF16 weights reads, for each fine cube near the
 * fluid boundary, a 4x4x4 patch of a coarse occupancy grid (cells of 2x2x2
 * fine cubes) and predicts whether the surface crosses the cube.  The field is
 * evaluated exactly at the band corners of the predicted cubes.  Every other
 * band vertex gets only a sign, which is exact: its walk stops as soon as a
 * partial sum of its (non-negative) terms exceeds iso (a sum over its nearest
 * cells first); a walk that never exceeds iso runs to the end and is the exact
 * value.  With every sign known, the marching-cubes classification of the
 * band is the plain band's; the certified corners of valid cubes are then
 * evaluated exactly, so the triangle soup equals the plain band's, whatever
 * the network predicted.  The network decides only which vertices are
 * evaluated exactly at once.
 * ------------------------------------------------------------------------- */
#define PMS_BAND_MLP_INPUTS 64
#define PMS_BAND_MLP_HIDDEN 64
#define PMS_BAND_MLP_PARAMS 4225          /* W1 64x64, b1 64, w2 64, b2 */
typedef struct pms_band_model {
    uint16_t w1[PMS_BAND_MLP_INPUTS * PMS_BAND_MLP_HIDDEN];  /* bf16 bits, w1[i * 64 + j]: input i -> hidden j */
    float b1[PMS_BAND_MLP_HIDDEN];
    uint16_t w2[PMS_BAND_MLP_HIDDEN];    /* bf16 bits */
    float b2;
    float threshold;                     /* a cube is predicted when its logit exceeds this */
} pms_band_model;

pms_status pms_set_band_model(pms_ctx* ctx, const pms_band_model* model);
/* Which band pms_run_frame uses: PMS_BAND_LEARNED needs a model; PMS_BAND_CERTIFIED
 * is the learned band's exact sign certification without the network (every band
 * vertex certified first).  A context created from a config naming [GB300]
 * BandModel starts in PMS_BAND_LEARNED.
 * Both give the plain band's triangle soup exactly (positions: what the PLY file
 * holds, FileData.cpp:1322-1327).  A vertex normal is a central difference of the
 * field at the neighbours of a valid cube's corners; where such a neighbour is a
 * certified vertex that is not itself a valid cube's corner, it reads the partial
 * sum (above iso) instead of the exact value, so the normals from
 * pms_download_mesh can differ slightly from the plain band's there. */
#define PMS_BAND_PLAIN 0
#define PMS_BAND_LEARNED 1
#define PMS_BAND_CERTIFIED 2
pms_status pms_set_band_mode(pms_ctx* ctx, int mode);
/* Model files: "PMSBAND1", uint32 version 1, uint32 sizeof(pms_band_model),
 * the struct (little-endian), uint32 length and that many bytes of JSON
 * metadata (training provenance). */
pms_status pms_save_band_model(const char* path, const pms_band_model* model, const char* meta_json);
pms_status pms_load_band_model(const char* path, pms_band_model* out);
/* Band and field in one: after pms_anisotropy; followed by pms_marching_cubes. */
pms_status pms_band_learned(pms_ctx* ctx);
/* pms_anisotropy + pms_band_learned + pms_marching_cubes. */
pms_status pms_surface_learned(pms_ctx* ctx);

/* Training data of the current frame, after a plain pms_surface: the coarse
 * grid, the candidate cubes and the plain method's labels (valid cubes). */
pms_status pms_learn_prepare(pms_ctx* ctx, uint32_t* n_candidates, uint32_t* n_valid_cubes);
/* Candidate cubes (origin vertex ids) with the logits of the context's model
 * and the plain labels; *n receives the count even when it exceeds cap. */
pms_status pms_learn_candidates(pms_ctx* ctx, uint32_t* cube_ids, float* logits, uint8_t* labels, uint32_t cap,
                                uint32_t* n);
/* Features (bf16 bits, 64 per cube) of the given cubes, after pms_learn_prepare. */
pms_status pms_learn_features(pms_ctx* ctx, const uint32_t* cube_ids, uint32_t n, uint16_t* x_bf16);

/* Trainer: fp32 master weights, Adam state, and the bf16 model the forward
 * pass reads; the forward and backward kernels run on the tensor cores. */
typedef struct pms_trainer pms_trainer;
pms_status pms_trainer_create(int device, uint64_t seed, pms_trainer** out);
void       pms_trainer_destroy(pms_trainer* t);
/* One Adam step on `batch` candidates sampled (by `seed`) from the frame that
 * pms_learn_prepare set up in `data`; *loss receives the batch's mean loss. */
pms_status pms_trainer_step(pms_trainer* t, pms_ctx* data, uint32_t batch, uint64_t seed, float lr, float pos_weight,
                            float* loss);
/* Gradient of the mean weighted cross-entropy over explicit samples, without
 * an update (grad: PMS_BAND_MLP_PARAMS floats in the parameter layout). */
pms_status pms_trainer_grad(pms_trainer* t, const uint16_t* x_bf16, const uint8_t* labels, uint32_t batch,
                            float pos_weight, float* grad, float* loss);
pms_status pms_trainer_get_params(pms_trainer* t, float* params);
pms_status pms_trainer_set_params(pms_trainer* t, const float* params);
/* The bf16 model of the current weights (threshold 0). */
pms_status pms_trainer_get_model(pms_trainer* t, pms_band_model* out);

/* ---------------------------------------------------------------------------
 * Batched frames.  No counterpart in the reference, whose GPUPOST::runSimulation
 * (GPUPOST.cpp:56-81) reconstructs one frame at a time with host round trips
 * between stages.  pms_run_batch copies k frames (host or device pointers) into
 * one device arena, finds their grids with one synchronisation, and runs the
 * surface path of all of them in one CUDA graph launch (captured on first use
 * and relaunched while the frames' grids stay the same).  When the context's
 * config has diffuse generation on, the frames are consecutive frames of one
 * sequence: each frame's diffuse stage runs inside the graph in frame order,
 * carrying the particles from frame to frame (starting from, and leaving, the
 * context's carried set and frame counter, so batches and single frames
 * continue one sequence); pms_batch_diffuse reads a frame's live particles.
 * With PMS_BATCH_LEARNED the learned band is used (PMS_BATCH_CERTIFIED: its
 * sign certification without the network); every frame's result equals its
 * single-frame run, and the plain band's.
 * ------------------------------------------------------------------------- */
typedef struct pms_frame {
    const float* pos_xyz;
    const float* vel_xyz;   /* may be NULL */
    const float* rhop;      /* may be NULL */
    uint32_t n;
} pms_frame;
#define PMS_BATCH_LEARNED 1
#define PMS_BATCH_CERTIFIED 2
pms_status pms_run_batch(pms_ctx* ctx, const pms_frame* frames, uint32_t k, int flags);
/* Counts of frame f of the last batch and its device time inside the graph. */
pms_status pms_batch_frame(pms_ctx* ctx, uint32_t f, pms_counts* counts, float* ms);
/* Triangle soup of frame f (positions, 3 vertices per triangle). */
pms_status pms_batch_mesh(pms_ctx* ctx, uint32_t f, float* pos_xyz, uint64_t cap, uint64_t* n_vertices);
/* Registers a page-locked host arena (cudaHostAlloc or cudaHostRegister memory,
 * mapped) of cap_vertices vertices that every following pms_run_batch fills inside
 * its graph: each frame's soup is stored there by the SMs right after the frame's
 * emission, on the frame's lane, while the other lanes compute.  Frame f's soup
 * starts at vertex pms_batch_mesh_range's *first (the layout of the device arena);
 * it has landed when pms_run_batch returns.  A batch whose meshes do not fit
 * returns PMS_ERR_CAPACITY.  pos_xyz NULL unregisters; the graph is captured again
 * when the registration changes.  No reference counterpart (its frames copy their
 * soup back one by one, FileData.cpp:1300-1305). */
pms_status pms_batch_stream_meshes(pms_ctx* ctx, float* pos_xyz, uint64_t cap_vertices);
/* First vertex and vertex count of frame f's soup in the last batch's arenas. */
pms_status pms_batch_mesh_range(pms_ctx* ctx, uint32_t f, uint64_t* first, uint64_t* n_vertices);
/* Live diffuse particles of frame f of the last batch (after its delete/append),
 * as the 32-byte records of pms_stream_diffuse_to_host; *n receives the count
 * (PMS_ERR_CAPACITY, with the count, when cap is too small; out NULL: count only). */
pms_status pms_batch_diffuse(pms_ctx* ctx, uint32_t f, pms_diffuse_particle* out, uint64_t cap, uint64_t* n);
/* Kernels per graph launch, graph captures so far. */
pms_status pms_batch_info(pms_ctx* ctx, uint32_t* graph_kernels, uint32_t* captures);

/* ---------------------------------------------------------------------------
 * Autotuner.  No counterpart in the reference (fixed launch shapes).  After a
 * reconstructed frame, pms_autotune times every candidate launch shape of the
 * neighbour walks on that frame -- threads per block 64/128/256 for density,
 * moments and field, and the field's cap of 1/2/4/8 resident waves of blocks --
 * keeps the fastest in the context (results do not depend on the shape) and
 * reports it.  pms_set_tune applies a shape chosen earlier (e.g. cached by
 * the caller per workload); batches use the context's shape.
 * ------------------------------------------------------------------------- */
typedef struct pms_tune {
    int field_threads, field_waves, density_threads, moments_threads;
    int field_vpt;                     /* band vertices per field work item: 1, 2 or 4 (x-neighbours) */
    float anisotropy_ms, field_ms;     /* the chosen shapes' times on the tuning frame */
} pms_tune;
pms_status pms_autotune(pms_ctx* ctx, pms_tune* out);
pms_status pms_set_tune(pms_ctx* ctx, const pms_tune* t);
pms_status pms_get_tune(pms_ctx* ctx, pms_tune* out);


/* Exclusive prefix sum of n uint32 device values into d_out (d_total, if not
 * NULL, receives the sum), on cuda_stream (NULL: the default stream).  It
 * allocates nothing -- for host programs that own all device memory or that
 * cannot afford cudaMalloc's implicit synchronisation inside a frame; its only
 * scratch is a 16 KiB file-scope device array held by every GPU that loads the
 * library.  n above 33,554,432 returns PMS_ERR_CAPACITY.  The first call on
 * each device looks up that array's device address (make it before any stream
 * capture).  Concurrent calls on the GPU share the scratch and race.
 * No counterpart in the reference (its scans allocate through thrust). */
pms_status pms_exclusive_scan_u32_noalloc(const uint32_t* d_in, uint32_t* d_out, uint64_t n, uint32_t* d_total,
                                          void* cuda_stream);

/* ---------------------------------------------------------------------------
 * File formats (host)
 * ------------------------------------------------------------------------- */
/* Legacy-VTK polydata particles (ASCII or BINARY, float or double points,
 * point arrays "Vel" and "Rhop", FileData.cpp:191-230).  Arrays are malloc'ed;
 * release with pms_free_host. */
pms_status pms_read_vtk_particles(const char* path, float** pos_xyz, float** vel_xyz, float** rhop, uint32_t* n);
/* Writes particles as BINARY legacy VTK polydata with Vel and Rhop arrays. */
pms_status pms_write_vtk_particles(const char* path, const float* pos_xyz, const float* vel_xyz,
                                   const float* rhop, uint32_t n);
/* Surface mesh with Normal (negated, as the reference writes it), Rhop, VelLength and
 * Vel point arrays, BINARY legacy VTK (FileData::saveSurfaceVTKfile, FileData.cpp:677-773). */
pms_status pms_write_surface_vtk(const char* path, const float* pos_xyz, const float* nrm_xyz, const float* vel_xyz,
                                 const float* vel_len, const float* rhop, uint64_t n_vertices);
/* ASCII PLY triangle soup in tinyply 2.3's layout (FileData.cpp:1277-1332). */
pms_status pms_write_ply(const char* path, const float* pos_xyz, uint64_t n_vertices);
/* PLY with a face list: indices NULL writes the soup (faces 3k, 3k+1, 3k+2), else
 * n_indices / 3 triangles over the n_vertices vertices; binary != 0 writes
 * binary_little_endian (12 bytes per vertex, 13 per face), else ASCII (9 significant
 * digits, so the float32 positions read back exactly).  The soup in ASCII is
 * pms_write_ply's layout. */
pms_status pms_write_ply_mesh(const char* path, const float* pos_xyz, uint64_t n_vertices, const uint32_t* indices,
                              uint64_t n_indices, int binary);
/* Diffuse particles as BINARY legacy VTK with Velocity, Size, energy, Ita and
 * waveCrest arrays (FileData.cpp:945-1036). */
pms_status pms_write_diffuse_vtk(const char* path, const float* pos_xyz, const float* vel_xyz,
                                 const float* energy, const float* ita, const float* wave_crest,
                                 uint32_t n, float size);
void pms_free_host(void* p);

/* The VisGPU program: reads config_path, then for each frame reads
 * FluidPath/FluidPrefix%0NNd.vtk, reconstructs, and writes
 * SurfacePath/SurfacePrefix%0NNd.ply and (diffuse on) the PartSpary_/PartFoam_/
 * PartBubble_ VTK files.  Replaces Main.cpp:4-11 / GPUPOST::runSimulation. */
pms_status pms_run_config(const char* config_path, int verbose);

#ifdef __cplusplus
}
#endif
#endif /* PMS_H */
