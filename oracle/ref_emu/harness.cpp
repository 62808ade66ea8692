/*
 * harness.cpp -- runs the reference's own CUDA kernels on the CPU
 * (TEST INFRASTRUCTURE: builds oracle/_ref/libref_emu.so, used only to pin the
 * oracle and to generate tests/golden fixtures; never shipped).
 *
 * The kernels (NeighborSearch_kernel.cuh, Anisotropic_kernel.cuh,
 * MarchingCube_kernel.cuh, SVD3.cuh, myCuda.cuh) and the parameter code
 * (Params.cpp with inih) are compiled unmodified from the reference tree; the
 * prelude in include/ maps the CUDA dialect to C++.  This file restates only
 * the host orchestration that drives them:
 *   FileData.cpp:239-279           bounding box and per-frame grid
 *   NeighborSearch.cu:37-76        hash, sort_by_key, cell ranges
 *   Anisotropic.cu:30-254          surface particles, anisotropy, band, field
 *   MarchingCube.cu:32-164         classify, scans, compaction, emit
 * thrust::sort_by_key (stable radix sort on uint keys) and
 * thrust::exclusive_scan are replaced by std::stable_sort and a serial scan.
 * Every "launch" runs the kernel body once per thread index, serially, with
 * blockDim = 1 so that shared-memory kernels see exactly their own data.
 */
#include "Params.h"
#include "MarchingCubesHelper.h"
#include "myCuda.cuh"
#include "NeighborSearch_kernel.cuh"
#include "Anisotropic_kernel.cuh"
#include "MarchingCube_kernel.cuh"
#include "DiffuseGeneration_kernel.cuh"

#include <vector>
#include <numeric>
#include <string>

thread_local dim3 threadIdx(0, 0, 0);
thread_local dim3 blockIdx(0, 0, 0);
thread_local dim3 blockDim(1, 1, 1);
thread_local dim3 gridDim(1, 1, 1);

/* Constants.cu:3-20 */
SimParams dSimParams;
SurfaceParams dSurfaceParams;
GridParams dGridParams;
DiffuseParams dDiffuseParams;
uint dNumSurfaceParticles, dNumInvolveParticles, dNumSurfaceVertices;
uint dNumFreeSurfaceParticles, dGeneratedNumDiffuseParticles, dNumIsDiffuseParticles;
uint dOldNumDiffuseParticles, dNumParticles, dNumValidSurfaceCubes, dNumSurfaceMeshVertices;

/* backing store for calCellRange's dynamic shared memory (blockDim == 1) */
unsigned int sharedHash[2];

template <class F>
static void launch(uint64_t n, F&& body)
{
    gridDim = dim3((unsigned)n, 1, 1);
    blockDim = dim3(1, 1, 1);
    threadIdx = dim3(0, 0, 0);
    for (uint64_t b = 0; b < n; ++b) { blockIdx = dim3((unsigned)b, 0, 0); body(); }
}

template <class T, class S>
static uint exclusive_scan(const T* in, S* out, uint64_t n)
{
    uint64_t acc = 0;
    for (uint64_t i = 0; i < n; ++i) { out[i] = (S)acc; acc += in[i]; }
    return (uint)acc;
}

template <class T>
static T* dup(const T* src, uint64_t count)
{
    T* p = (T*)std::malloc(sizeof(T) * (count ? count : 1));
    if (count) std::memcpy(p, src, sizeof(T) * count);
    return p;
}

extern "C" {

/* All arrays are owned by the harness until ref_free(). */
struct ref_result {
    /* grid */
    float min_pos[3], max_pos[3], scmin_pos[3], scmax_pos[3];
    float sp_grid_size, sc_grid_size;
    uint32_t spres[3], scres[3];
    int32_t spexpand, scexpand;
    uint32_t sp_size, sc_size;
    /* derived surface params */
    float h, h_inv, h_sq, aniso_radius, iso, mass;
    int32_t min_nn;
    /* counts */
    uint32_t n, n_surface, n_band, n_valid, n_mesh;
    /* per particle, in sorted order */
    uint32_t* keys_sorted;   /* n */
    uint32_t* perm;          /* n: input index of sorted slot */
    float* pos_sorted;       /* 3n */
    float* rho;              /* n (density written by calculationOfDensity) */
    float* nrm;              /* 3n (normals of surface particles, 0 elsewhere) */
    float* flag;             /* n */
    /* per spatial cell */
    uint32_t* cell_start;    /* sp_size */
    uint32_t* cell_end;      /* sp_size */
    uint32_t* surf_count;    /* sp_size: numSurParticleGrid */
    /* per surface particle */
    uint32_t* surf_list;     /* n_surface */
    float* mean;             /* 3 n_surface */
    float* G;                /* 10 n_surface (MatrixValue: 9 + maxvalue) */
    /* scalar grid */
    uint32_t* band_flags;    /* sc_size (0/1) */
    uint32_t* band_list;     /* n_band */
    float* field;            /* n_band: field at band vertices */
    uint32_t* cube_flag;     /* n_band */
    uint32_t* nvert;         /* n_band */
    float* vpos;             /* 3 n_mesh */
    float* vnrm;             /* 3 n_mesh */
    float* sval;             /* 5 n_mesh: ScalarValue {vel xyz, |vel|, rhop} (estimationOfScalarValue) */
};

void ref_free(ref_result* r)
{
    void* ptrs[] = {r->keys_sorted, r->perm, r->pos_sorted, r->rho, r->nrm, r->flag, r->cell_start, r->cell_end,
                    r->surf_count, r->surf_list, r->mean, r->G, r->band_flags, r->band_list, r->field,
                    r->cube_flag, r->nvert, r->vpos, r->vnrm, r->sval};
    for (void* p : ptrs) std::free(p);
    std::memset(r, 0, sizeof(*r));
}

/* Runs one frame of the reference's plain surface path.  config_path is a
 * reference config.txt (read by the reference's own Params::setParams). */
int ref_surface_run(const char* config_path, const float* pos, const float* vel, const float* rhop,
                    uint32_t n, ref_result* out)
{
    std::memset(out, 0, sizeof(*out));
    if (n == 0) return 1;
    Params params;
    params.mConfigParams.FileName_Param = config_path;
    params.setParams();

    /* FileData.cpp:214-257: particles and bounding box (motion = 0) */
    std::vector<FluidParticle> fp(n);
    for (uint32_t i = 0; i < n; ++i) {
        FluidParticle p;
        std::memset(&p, 0, sizeof(p));
        p.pos = make_float3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        p.vel = make_float3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        p.rhop = rhop[i];
        fp[i] = p;
    }
    float3 mx = fp[0].pos, mn = fp[0].pos;
    for (uint32_t i = 1; i < n; ++i) {
        if (mx.x <= fp[i].pos.x) mx.x = fp[i].pos.x;
        if (mx.y <= fp[i].pos.y) mx.y = fp[i].pos.y;
        if (mx.z <= fp[i].pos.z) mx.z = fp[i].pos.z;
        if (mn.x >= fp[i].pos.x) mn.x = fp[i].pos.x;
        if (mn.y >= fp[i].pos.y) mn.y = fp[i].pos.y;
        if (mn.z >= fp[i].pos.z) mn.z = fp[i].pos.z;
    }
    /* FileData.cpp:259-279 */
    GridParams& g = params.mGridParams;
    g.scminPos = mn - 2 * params.mSurfaceParams.smoothingRadius;
    g.scmaxPos = mx + 2 * params.mSurfaceParams.smoothingRadius;
    g.minPos = mn - 4 * params.mSurfaceParams.smoothingRadius;
    g.maxPos = mx + 4 * params.mSurfaceParams.smoothingRadius;
    g.spresolution = make_uint3(
        (uint)((g.maxPos.x - g.minPos.x) / g.spGridSize),
        (uint)((g.maxPos.y - g.minPos.y) / g.spGridSize),
        (uint)((g.maxPos.z - g.minPos.z) / g.spGridSize));
    g.scresolution = make_uint3(
        (uint)(((g.scmaxPos.x - g.scminPos.x) / g.scGridSize) + 0.5),
        (uint)(((g.scmaxPos.y - g.scminPos.y) / g.scGridSize) + 0.5),
        (uint)(((g.scmaxPos.z - g.scminPos.z) / g.scGridSize) + 0.5));
    g.spSize = g.spresolution.x * g.spresolution.y * g.spresolution.z;
    g.scSize = g.scresolution.x * g.scresolution.y * g.scresolution.z;

    dSimParams = params.mSimParams;
    dSurfaceParams = params.mSurfaceParams;
    dGridParams = g;
    const uint spSize = g.spSize, scSize = g.scSize;

    /* GPUmemory.cpp:47-72 */
    std::vector<SpatialGrid> spatialGrid(spSize);
    std::memset(spatialGrid.data(), 0, sizeof(SpatialGrid) * spSize);
    std::vector<IndexRange> range(spSize, IndexRange{0, 0});
    std::vector<uint> numSur(spSize, 0), numInv(spSize, 0), numSurScan(spSize, 0);
    std::vector<ScalarFieldGrid> field(scSize, 0.0f);
    std::vector<IsSurface> isSV(scSize, 0);
    std::vector<IsSurfaceScan> isSVScan(scSize, 0);

    /* NeighborSearch.cu:37-76 */
    std::vector<uint> hash(n);
    FluidParticle* P = fp.data();
    launch(n, [&] { calculateHash(hash.data(), P, n, spatialGrid.data()); });
    std::vector<uint> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint a, uint b) { return hash[a] < hash[b]; });
    std::vector<FluidParticle> sorted(n);
    std::vector<uint> skeys(n);
    for (uint i = 0; i < n; ++i) { sorted[i] = fp[order[i]]; skeys[i] = hash[order[i]]; }
    fp.swap(sorted);
    P = fp.data();
    launch(n, [&] { calCellRange(range.data(), n, skeys.data(), P); });

    out->n = n;
    out->keys_sorted = dup(skeys.data(), n);
    out->perm = dup(order.data(), n);
    std::memcpy(out->min_pos, &g.minPos, 12); std::memcpy(out->max_pos, &g.maxPos, 12);
    std::memcpy(out->scmin_pos, &g.scminPos, 12); std::memcpy(out->scmax_pos, &g.scmaxPos, 12);
    out->sp_grid_size = g.spGridSize; out->sc_grid_size = g.scGridSize;
    std::memcpy(out->spres, &g.spresolution, 12); std::memcpy(out->scres, &g.scresolution, 12);
    out->spexpand = g.spexpandExtent; out->scexpand = g.scexpandExtent;
    out->sp_size = spSize; out->sc_size = scSize;
    out->h = dSurfaceParams.smoothingRadius; out->h_inv = dSurfaceParams.smoothingRadiusInv;
    out->h_sq = dSurfaceParams.smoothingRadiusSq; out->aniso_radius = dSurfaceParams.anisotropicRadius;
    out->iso = dSurfaceParams.isoValue; out->mass = dSimParams.mass; out->min_nn = dSurfaceParams.minNumNeighbors;
    out->cell_start = (uint32_t*)std::malloc(4 * (size_t)spSize);
    out->cell_end = (uint32_t*)std::malloc(4 * (size_t)spSize);
    for (uint c = 0; c < spSize; ++c) { out->cell_start[c] = range[c].start; out->cell_end[c] = range[c].end; }

    /* Anisotropic.cu:30-40 processingOfParticles */
    launch(spSize, [&] { estimationOfSurfaceParticles(spatialGrid.data(), numSur.data(), numInv.data(), range.data()); });
    uint NumSurfaceParticles = exclusive_scan(numSur.data(), numSurScan.data(), spSize);
    out->surf_count = dup(numSur.data(), spSize);
    out->n_surface = NumSurfaceParticles;
    auto finish_particles = [&] {
        out->pos_sorted = (float*)std::malloc(12 * (size_t)n);
        out->rho = (float*)std::malloc(4 * (size_t)n);
        out->nrm = (float*)std::malloc(12 * (size_t)n);
        out->flag = (float*)std::malloc(4 * (size_t)n);
        for (uint i = 0; i < n; ++i) {
            std::memcpy(out->pos_sorted + 3 * i, &fp[i].pos, 12);
            out->rho[i] = fp[i].rhop;
            std::memcpy(out->nrm + 3 * i, &fp[i].nor, 12);
            out->flag[i] = fp[i].flag;
        }
    };
    if (NumSurfaceParticles == 0) { finish_particles(); return 2; }
    dNumSurfaceParticles = NumSurfaceParticles;
    dNumInvolveParticles = 0;
    std::vector<Index> surfIdx(NumSurfaceParticles, 0);
    std::vector<SmoothedPos> smoothed(NumSurfaceParticles);
    std::vector<MeanPos> meanP(NumSurfaceParticles);
    std::vector<MatrixValue> svd(NumSurfaceParticles);
    std::memset(smoothed.data(), 0, sizeof(SmoothedPos) * NumSurfaceParticles);
    std::memset(meanP.data(), 0, sizeof(MeanPos) * NumSurfaceParticles);
    std::memset(svd.data(), 0, sizeof(MatrixValue) * NumSurfaceParticles);
    launch(spSize, [&] { compactationOfParticles(numSur.data(), numSurScan.data(), range.data(), surfIdx.data()); });
    launch(NumSurfaceParticles, [&] { calculationOfSmoothed(P, meanP.data(), smoothed.data(), range.data(), surfIdx.data(), spatialGrid.data()); });
    launch(n, [&] { calculationOfDensity(P, range.data(), spatialGrid.data(), n); });
    launch(NumSurfaceParticles, [&] { calculationOfTransformMatrices(meanP.data(), P, range.data(), surfIdx.data(), svd.data()); });
    out->surf_list = dup(surfIdx.data(), NumSurfaceParticles);
    out->mean = (float*)std::malloc(12 * (size_t)NumSurfaceParticles);
    out->G = (float*)std::malloc(40 * (size_t)NumSurfaceParticles);
    for (uint s = 0; s < NumSurfaceParticles; ++s) {
        std::memcpy(out->mean + 3 * s, &meanP[s].pos, 12);
        std::memcpy(out->G + 10 * s, &svd[s], 40);
    }

    /* Anisotropic.cu:43-50 processingOfVertices */
    launch(NumSurfaceParticles, [&] {
        estimationOfSurfaceVertices(P, smoothed.data(), range.data(), surfIdx.data(), isSV.data(), svd.data(),
                                    spatialGrid.data(), field.data());
    });
    uint NumSurfaceVertices = exclusive_scan(isSV.data(), isSVScan.data(), scSize);
    out->band_flags = dup(isSV.data(), scSize);
    out->n_band = NumSurfaceVertices;
    if (NumSurfaceVertices == 0) { finish_particles(); return 3; }
    dNumSurfaceVertices = NumSurfaceVertices;
    std::vector<Index> svIndex(NumSurfaceVertices, 0);
    launch(scSize, [&] { compactationOfSurfaceVertices(isSV.data(), isSVScan.data(), svIndex.data()); });

    /* Anisotropic.cu:233-254 */
    launch(NumSurfaceVertices, [&] {
        computationOfScalarFieldGrid(P, smoothed.data(), nullptr, range.data(), surfIdx.data(), nullptr, svIndex.data(),
                                     numSur.data(), numSurScan.data(), numInv.data(), nullptr, svd.data(), field.data());
    });
    out->band_list = dup(svIndex.data(), NumSurfaceVertices);
    out->field = (float*)std::malloc(4 * (size_t)NumSurfaceVertices);
    for (uint v = 0; v < NumSurfaceVertices; ++v) out->field[v] = field[svIndex[v]];
    finish_particles();

    /* MarchingCube.cu:32-151 with the texture tables of MarchingCubesHelper.cpp */
    edgeTex.ptr = &MarchingCubesHelper::edgeFlags[0];
    edgeIndexesOfTriangleTex.ptr = &MarchingCubesHelper::edgeIndexesOfTriangle[0][0];
    numVerticesTex.ptr = &MarchingCubesHelper::numVertices[0];
    vertexIndexesOfEdgeTex.ptr = &MarchingCubesHelper::vertexIndexesOfEdge[0][0];
    std::vector<IsValid> isValid(NumSurfaceVertices, 0);
    std::vector<IsValidScan> isValidScan(NumSurfaceVertices, 0);
    std::vector<NumVertexCube> nVC(NumSurfaceVertices, 0);
    std::vector<NumVertexCubeScan> nVCScan(NumSurfaceVertices, 0);
    std::vector<CubeFlag> cubeFlag(NumSurfaceVertices, 0);
    launch(NumSurfaceVertices, [&] {
        detectValidSurfaceCubes(svIndex.data(), field.data(), isSV.data(), cubeFlag.data(), isValid.data(), nVC.data());
    });
    uint NumValid = exclusive_scan(isValid.data(), isValidScan.data(), NumSurfaceVertices);
    uint NumMesh = exclusive_scan(nVC.data(), nVCScan.data(), NumSurfaceVertices);
    out->cube_flag = dup(cubeFlag.data(), NumSurfaceVertices);
    out->nvert = dup(nVC.data(), NumSurfaceVertices);
    out->n_valid = NumValid;
    out->n_mesh = NumMesh;
    if (NumValid == 0 || NumMesh == 0) return 4;
    dNumValidSurfaceCubes = NumValid;
    dNumSurfaceMeshVertices = NumMesh;
    std::vector<Index> validIdx(NumValid, 0);
    std::vector<Vertex> vert(NumMesh);
    std::vector<Normal> norm(NumMesh);
    launch(NumSurfaceVertices, [&] { compactValidSurfaceCubes(validIdx.data(), isValid.data(), isValidScan.data()); });
    launch(NumValid, [&] {
        generateTriangles(svIndex.data(), validIdx.data(), cubeFlag.data(), nVCScan.data(), field.data(), vert.data(), norm.data());
    });
    out->vpos = (float*)std::malloc(12 * (size_t)NumMesh);
    out->vnrm = (float*)std::malloc(12 * (size_t)NumMesh);
    std::memcpy(out->vpos, vert.data(), 12 * (size_t)NumMesh);
    std::memcpy(out->vnrm, norm.data(), 12 * (size_t)NumMesh);
    /* MarchingCube.cu:50-52, 153-163: scalar values at the mesh vertices */
    std::vector<ScalarValue> sv(NumMesh);
    std::memset(sv.data(), 0, sizeof(ScalarValue) * NumMesh);
    launch(NumMesh, [&] { estimationOfScalarValue(vert.data(), P, range.data(), sv.data()); });
    out->sval = (float*)std::malloc(sizeof(ScalarValue) * (size_t)NumMesh);
    std::memcpy(out->sval, sv.data(), sizeof(ScalarValue) * (size_t)NumMesh);
    return 0;
}

/* Copies of the reference's marching-cubes tables, for the oracle's own MC
 * restatement in the test harness (MarchingCubesHelper.cpp:3-587). */
void ref_mc_tables(uint32_t* edge_flags, int32_t* tri, uint32_t* num_vertices, uint32_t* edge_vertices)
{
    std::memcpy(edge_flags, MarchingCubesHelper::edgeFlags, 256 * 4);
    std::memcpy(tri, MarchingCubesHelper::edgeIndexesOfTriangle, 256 * 16 * 4);
    std::memcpy(num_vertices, MarchingCubesHelper::numVertices, 256 * 4);
    std::memcpy(edge_vertices, MarchingCubesHelper::vertexIndexesOfEdge, 24 * 4);
}

/* ------------------------------------------------------------------------- */
/* diffuse particles: DiffuseGeneration::runsimulation (DiffuseGeneration.cu:89-104) */
/* ------------------------------------------------------------------------- */
struct ref_diffuse_result {
    uint32_t n, n_free, n_spawning, n_generated, n_old, n_live;
    uint32_t* perm;            /* n */
    uint32_t* free_list;       /* n_free */
    float* nrm;                /* 3n: particle normals after calculationofNormal */
    float* pot;                /* 3n: waveCrest, Ita, energy after the phi clamps */
    int32_t* num;              /* n */
    float* gen;                /* 8 n_generated: pos xyz, vel xyz, ttl, type */
    float* old_after;          /* 8 n_old: the old particles after updateDiffuseParticle */
    float* live;               /* 8 n_live: generated then old, type 3 removed */
};

void ref_diffuse_free(ref_diffuse_result* r)
{
    void* ptrs[] = {r->perm, r->free_list, r->nrm, r->pot, r->num, r->gen, r->old_after, r->live};
    for (void* p : ptrs) std::free(p);
    std::memset(r, 0, sizeof(*r));
}

static void pack_diffuse(const DiffuseParticle& d, float* o)
{
    o[0] = d.pos.x; o[1] = d.pos.y; o[2] = d.pos.z;
    o[3] = d.vel.x; o[4] = d.vel.y; o[5] = d.vel.z;
    o[6] = (float)d.TTL; o[7] = (float)d.type;
}

/* One frame.  `uniforms(3 * idif + k)` replaces the host mt19937 stream
 * (DiffuseGeneration.cu:381-395); old particles are given as 8-float records
 * (pos, vel, ttl, type).  With run_surface the surface path's anisotropy runs
 * first, as in GPUPOST.cpp:65-71, leaving its normals on surface particles. */
int ref_diffuse_frame(const char* config_path, const float* pos, const float* vel, const float* rhop, uint32_t n,
                      int run_surface, const float* old_rec, uint32_t n_old, const float* uniforms, uint64_t n_uniforms,
                      ref_diffuse_result* out)
{
    std::memset(out, 0, sizeof(*out));
    if (n == 0) return 1;
    Params params;
    params.mConfigParams.FileName_Param = config_path;
    params.setParams();
    std::vector<FluidParticle> fp(n);
    for (uint32_t i = 0; i < n; ++i) {
        FluidParticle p;
        std::memset(&p, 0, sizeof(p));
        p.pos = make_float3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        p.vel = make_float3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        p.rhop = rhop[i];
        fp[i] = p;
    }
    float3 mx = fp[0].pos, mn = fp[0].pos;
    for (uint32_t i = 1; i < n; ++i) {
        if (mx.x <= fp[i].pos.x) mx.x = fp[i].pos.x;
        if (mx.y <= fp[i].pos.y) mx.y = fp[i].pos.y;
        if (mx.z <= fp[i].pos.z) mx.z = fp[i].pos.z;
        if (mn.x >= fp[i].pos.x) mn.x = fp[i].pos.x;
        if (mn.y >= fp[i].pos.y) mn.y = fp[i].pos.y;
        if (mn.z >= fp[i].pos.z) mn.z = fp[i].pos.z;
    }
    GridParams& g = params.mGridParams;
    g.scminPos = mn - 2 * params.mSurfaceParams.smoothingRadius;
    g.scmaxPos = mx + 2 * params.mSurfaceParams.smoothingRadius;
    g.minPos = mn - 4 * params.mSurfaceParams.smoothingRadius;
    g.maxPos = mx + 4 * params.mSurfaceParams.smoothingRadius;
    g.spresolution = make_uint3((uint)((g.maxPos.x - g.minPos.x) / g.spGridSize),
                                (uint)((g.maxPos.y - g.minPos.y) / g.spGridSize),
                                (uint)((g.maxPos.z - g.minPos.z) / g.spGridSize));
    g.scresolution = make_uint3((uint)(((g.scmaxPos.x - g.scminPos.x) / g.scGridSize) + 0.5),
                                (uint)(((g.scmaxPos.y - g.scminPos.y) / g.scGridSize) + 0.5),
                                (uint)(((g.scmaxPos.z - g.scminPos.z) / g.scGridSize) + 0.5));
    g.spSize = g.spresolution.x * g.spresolution.y * g.spresolution.z;
    g.scSize = g.scresolution.x * g.scresolution.y * g.scresolution.z;
    dSimParams = params.mSimParams;
    dSurfaceParams = params.mSurfaceParams;
    dDiffuseParams = params.mDiffuseParams;
    dGridParams = g;
    const uint spSize = g.spSize;
    std::vector<SpatialGrid> spatialGrid(spSize);
    std::memset(spatialGrid.data(), 0, sizeof(SpatialGrid) * spSize);
    std::vector<IndexRange> range(spSize, IndexRange{0, 0});
    /* NeighborSearch.cu:37-76 */
    std::vector<uint> hash(n);
    FluidParticle* P = fp.data();
    launch(n, [&] { calculateHash(hash.data(), P, n, spatialGrid.data()); });
    std::vector<uint> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint a, uint b) { return hash[a] < hash[b]; });
    std::vector<FluidParticle> sorted(n);
    std::vector<uint> skeys(n);
    for (uint i = 0; i < n; ++i) { sorted[i] = fp[order[i]]; skeys[i] = hash[order[i]]; }
    fp.swap(sorted);
    P = fp.data();
    launch(n, [&] { calCellRange(range.data(), n, skeys.data(), P); });
    out->n = n;
    out->perm = dup(order.data(), n);
    if (run_surface) {
        /* Anisotropic::processingOfParticles: leaves normals and flags on surface particles */
        std::vector<uint> numSur(spSize, 0), numInv(spSize, 0), numSurScan(spSize, 0);
        launch(spSize, [&] { estimationOfSurfaceParticles(spatialGrid.data(), numSur.data(), numInv.data(), range.data()); });
        uint ns = exclusive_scan(numSur.data(), numSurScan.data(), spSize);
        if (ns) {
            dNumSurfaceParticles = ns;
            std::vector<Index> surfIdx(ns, 0);
            std::vector<SmoothedPos> smoothed(ns);
            std::vector<MeanPos> meanP(ns);
            std::vector<MatrixValue> svd(ns);
            std::memset(meanP.data(), 0, sizeof(MeanPos) * ns);
            launch(spSize, [&] { compactationOfParticles(numSur.data(), numSurScan.data(), range.data(), surfIdx.data()); });
            launch(ns, [&] { calculationOfSmoothed(P, meanP.data(), smoothed.data(), range.data(), surfIdx.data(), spatialGrid.data()); });
            launch(n, [&] { calculationOfDensity(P, range.data(), spatialGrid.data(), n); });
            launch(ns, [&] { calculationOfTransformMatrices(meanP.data(), P, range.data(), surfIdx.data(), svd.data()); });
        }
    }
    /* processingOfFreesurface (DiffuseGeneration.cu:187-198) */
    dNumParticles = n;
    std::vector<IsSurface> isFree(n, 0);
    std::vector<IsSurfaceScan> isFreeScan(n, 0);
    launch(spSize, [&] { estimationOfFreeSurfaceParticles(spatialGrid.data(), isFree.data(), range.data()); });
    uint nFree = exclusive_scan(isFree.data(), isFreeScan.data(), n);
    dNumFreeSurfaceParticles = nFree;
    std::vector<Index> freeIdx(nFree ? nFree : 1, 0);
    launch(n, [&] { compactationOfFreeParticles(isFree.data(), isFreeScan.data(), freeIdx.data()); });
    launch(nFree, [&] { calculationofNormal(P, range.data(), freeIdx.data()); });
    out->n_free = nFree;
    out->free_list = dup(freeIdx.data(), nFree);
    /* estimatingOfPotention (DiffuseGeneration.cu:200-212) */
    std::vector<DiffusePotential> pot(n);
    std::memset(pot.data(), 0, sizeof(DiffusePotential) * n);
    std::vector<IsDiffuse> isDiff(n, 0);
    std::vector<IsDiffuseScan> isDiffScan(n, 0);
    std::vector<NumDiffuseParticle> num(n, 0);
    std::vector<NumDiffuseParticleScan> numScan(n, 0);
    launch(n, [&] { calculationofTrappedairpotential(P, range.data(), pot.data()); });
    launch(nFree, [&] { calculationofWavecrests(P, range.data(), freeIdx.data(), pot.data()); });
    out->nrm = (float*)std::malloc(12 * (size_t)n);
    for (uint i = 0; i < n; ++i) std::memcpy(out->nrm + 3 * i, &fp[i].nor, 12);
    /* generatingOfDiffuse (DiffuseGeneration.cu:214-228) */
    launch(n, [&] { calculateofNumberofdiffuseparticles(pot.data(), num.data(), isDiff.data()); });
    out->pot = (float*)std::malloc(12 * (size_t)n);
    for (uint i = 0; i < n; ++i) { out->pot[3 * i] = pot[i].waveCrest; out->pot[3 * i + 1] = pot[i].Ita; out->pot[3 * i + 2] = pot[i].energy; }
    out->num = dup(num.data(), n);
    uint nGen = 0;
    { uint64_t acc = 0; for (uint i = 0; i < n; ++i) { numScan[i] = (uint)acc; acc += (uint)num[i]; } nGen = (uint)acc; }
    uint nSpawn = exclusive_scan(isDiff.data(), isDiffScan.data(), n);
    dGeneratedNumDiffuseParticles = nGen;
    dNumIsDiffuseParticles = nSpawn;
    out->n_spawning = nSpawn;
    out->n_generated = nGen;
    std::vector<Index> diffIdx(nSpawn ? nSpawn : 1, 0);
    std::vector<DiffuseParticle> gen(nGen ? nGen : 1);
    std::memset(gen.data(), 0, sizeof(DiffuseParticle) * gen.size());
    launch(n, [&] { compactationOfDiffuseParticle(isDiff.data(), isDiffScan.data(), diffIdx.data()); });
    if (nGen && (uint64_t)3 * nGen > n_uniforms) return 5;
    std::vector<float> rnd(uniforms, uniforms + (size_t)3 * nGen);
    launch(nSpawn, [&] { calculateofDiffusePosition(P, num.data(), numScan.data(), gen.data(), rnd.data(), pot.data(), diffIdx.data()); });
    launch(nGen, [&] { calculateofDiffuseType(P, range.data(), gen.data(), spatialGrid.data()); });
    out->gen = (float*)std::malloc(32 * (size_t)(nGen ? nGen : 1));
    for (uint k = 0; k < nGen; ++k) pack_diffuse(gen[k], out->gen + 8 * k);
    /* updatingOfDiffuse (DiffuseGeneration.cu:426-442) */
    std::vector<DiffuseParticle> old(n_old ? n_old : 1);
    std::memset(old.data(), 0, sizeof(DiffuseParticle) * old.size());
    for (uint k = 0; k < n_old; ++k) {
        const float* o = old_rec + 8 * (size_t)k;
        old[k].pos = make_float3(o[0], o[1], o[2]);
        old[k].vel = make_float3(o[3], o[4], o[5]);
        old[k].TTL = (int)o[6];
        old[k].type = (int)o[7];
        old[k].life = 1;
    }
    dOldNumDiffuseParticles = n_old;
    if (n_old) launch(n_old, [&] { updateDiffuseParticle(P, range.data(), old.data(), spatialGrid.data()); });
    out->n_old = n_old;
    out->old_after = (float*)std::malloc(32 * (size_t)(n_old ? n_old : 1));
    for (uint k = 0; k < n_old; ++k) pack_diffuse(old[k], out->old_after + 8 * k);
    /* deleteAndappendParticles (DiffuseGeneration.cu:760-867): generated, then old; type 3 dropped */
    std::vector<float> live;
    for (uint k = 0; k < nGen; ++k) if (gen[k].type != 3) { float r[8]; pack_diffuse(gen[k], r); live.insert(live.end(), r, r + 8); }
    for (uint k = 0; k < n_old; ++k) if (old[k].type != 3) { float r[8]; pack_diffuse(old[k], r); live.insert(live.end(), r, r + 8); }
    out->n_live = (uint32_t)(live.size() / 8);
    out->live = dup(live.data(), live.size());
    return 0;
}

} /* extern "C" */
