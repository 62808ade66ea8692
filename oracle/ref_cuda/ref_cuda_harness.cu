/*
 * ref_cuda_harness.cu -- times the reference's own CUDA code on this GPU
 * (BASELINE TIMING ONLY: baseline/_ref/libref_cuda.so, loaded by bench.py;
 * never part of libpms).
 *
 * The reference's sources (GPUPOST.cpp, GPUmemory.cpp, Params.cpp and the
 * NeighborSearch, Anisotropic, MarchingCube, SurfaceReconstruction,
 * DiffuseGeneration and Constants .cu files with their kernel headers) are
 * compiled unmodified for sm_103a; include/ref_cuda_prelude.h maps their
 * texture references to device pointers and include/FileData.h replaces the
 * VTK-based file layer.  This file implements that replacement:
 *   loadFluidFile    the frame comes from memory (the harness's arrays) instead
 *                    of a VTK file; bounding box and per-frame grid are the
 *                    reference's (FileData.cpp:239-283, NOBOUND on), restated;
 *                    then gMemory->memAlcandCpy_fluid, as the reference does;
 *   saveSurfacePLYfile  the mesh's positions and normals are copied back to the
 *                    host as the reference does (FileData.cpp:1279-1305); the
 *                    ASCII PLY text is not written;
 *   saveDiffuseVTKfile  the particles (already on the host) are counted, no file.
 * ref_cuda_run() then runs GPUPOST::initialize / runSimulation / finalize on
 * frames Framefrom..Frameto of the config.txt in the working directory and
 * returns the wall time per frame.
 */
#include <chrono>
#include <cstring>
#include <iostream>
#include <streambuf>
#include <vector>

#include "FileData.h"
#include "GPUPOST.h"

namespace {
const float* g_pos = nullptr;
const float* g_vel = nullptr;
const float* g_rho = nullptr;
uint32_t g_n = 0;
uint64_t g_mesh_vertices = 0;
uint64_t g_diffuse[3] = {0, 0, 0};
std::vector<Vertex> g_positions;
std::vector<Normal> g_normals;

struct NullBuf : std::streambuf {
    int overflow(int c) override { return c; }
};
}  // namespace

FileData::FileData(Params* p, GPUmemory* m) : params(p), gMemory(m) {}

void FileData::loadFluidFile(int idx, float3& motion) {
    frameIndex = idx;
    std::vector<FluidParticle> fp(g_n);
    for (uint32_t i = 0; i < g_n; ++i) {
        FluidParticle q;
        std::memset(&q, 0, sizeof(q));
        q.pos = make_float3(g_pos[3 * i], g_pos[3 * i + 1], g_pos[3 * i + 2]) - motion;
        q.vel = g_vel ? make_float3(g_vel[3 * i], g_vel[3 * i + 1], g_vel[3 * i + 2]) : make_float3(0.f, 0.f, 0.f);
        q.rhop = g_rho ? g_rho[i] : 0.f;
        fp[i] = q;
    }
    // bounding box, then the grid around it (FileData.cpp:239-279, NOBOUND)
    float3 mx = fp[0].pos, mn = fp[0].pos;
    for (uint32_t i = 1; i < g_n; ++i) {
        if (mx.x <= fp[i].pos.x) mx.x = fp[i].pos.x;
        if (mx.y <= fp[i].pos.y) mx.y = fp[i].pos.y;
        if (mx.z <= fp[i].pos.z) mx.z = fp[i].pos.z;
        if (mn.x >= fp[i].pos.x) mn.x = fp[i].pos.x;
        if (mn.y >= fp[i].pos.y) mn.y = fp[i].pos.y;
        if (mn.z >= fp[i].pos.z) mn.z = fp[i].pos.z;
    }
    GridParams& g = params->mGridParams;
    const float h = params->mSurfaceParams.smoothingRadius;
    g.scminPos = mn - 2 * h;
    g.scmaxPos = mx + 2 * h;
    g.minPos = mn - 4 * h;
    g.maxPos = mx + 4 * h;
    g.spresolution = make_uint3((g.maxPos.x - g.minPos.x) / g.spGridSize, (g.maxPos.y - g.minPos.y) / g.spGridSize,
                                (g.maxPos.z - g.minPos.z) / g.spGridSize);
    g.scresolution = make_uint3(((g.scmaxPos.x - g.scminPos.x) / g.scGridSize) + 0.5,
                                ((g.scmaxPos.y - g.scminPos.y) / g.scGridSize) + 0.5,
                                ((g.scmaxPos.z - g.scminPos.z) / g.scGridSize) + 0.5);
    g.spSize = g.spresolution.x * g.spresolution.y * g.spresolution.z;
    g.scSize = g.scresolution.x * g.scresolution.y * g.scresolution.z;
    gMemory->memAlcandCpy_fluid(fp);
}

void FileData::saveSurfacePLYfile() {
    const size_t m = gMemory->NumSurfaceMeshVertices;
    g_mesh_vertices = m;
    g_positions.resize(m);
    g_normals.resize(m);
    checkCudaErrors(cudaMemcpy(static_cast<void*>(g_positions.data()), gMemory->dVertex, sizeof(Vertex) * m,
                               cudaMemcpyDeviceToHost));
    checkCudaErrors(cudaMemcpy(static_cast<void*>(g_normals.data()), gMemory->dNormal, sizeof(Normal) * m,
                               cudaMemcpyDeviceToHost));
}

void FileData::saveDiffuseVTKfile(std::vector<DiffuseParticle> diffuse, uint type) {
    if (type < 3) g_diffuse[type] = diffuse.size();
}

extern "C" {

struct ref_cuda_result {
    double seconds_per_frame;      // wall time of GPUPOST::runSimulation / frames
    uint64_t mesh_vertices;        // of the last frame
    uint64_t spray, foam, bubble;  // of the last frame
    int frames;
};

// Runs the reference on `frames` copies of one frame (config.txt in the working
// directory must name Framefrom 0 .. Frameto frames - 1).  quiet: the reference's
// console output is dropped.
int ref_cuda_run(const float* pos, const float* vel, const float* rho, uint32_t n, int frames, int quiet,
                 ref_cuda_result* out) {
    if (!pos || n == 0 || frames < 1 || !out) return 1;
    g_pos = pos; g_vel = vel; g_rho = rho; g_n = n;
    NullBuf null;
    std::streambuf* old = quiet ? std::cout.rdbuf(&null) : nullptr;
    GPUPOST post;
    post.initialize();
    const auto t0 = std::chrono::steady_clock::now();
    post.runSimulation();
    checkCudaErrors(cudaDeviceSynchronize());
    const auto t1 = std::chrono::steady_clock::now();
    post.finalize();
    if (old) std::cout.rdbuf(old);
    out->seconds_per_frame = std::chrono::duration<double>(t1 - t0).count() / frames;
    out->mesh_vertices = g_mesh_vertices;
    out->spray = g_diffuse[0];
    out->foam = g_diffuse[1];
    out->bubble = g_diffuse[2];
    out->frames = frames;
    return 0;
}

}  // extern "C"
