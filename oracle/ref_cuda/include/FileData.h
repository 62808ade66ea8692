/*
 * FileData stand-in for the reference's CUDA build (baseline timing only).
 *
 * The reference's FileData (FileData.h / FileData.cpp) reads legacy VTK frames
 * through the VTK library and writes PLY / VTK files; neither VTK nor file I/O
 * belongs in the timing.  This class keeps the members the compiled reference
 * sources call -- GPUPOST::runSimulation's loadFluidFile (GPUPOST.cpp:58),
 * SurfaceReconstruction::runsimulation's saveSurfacePLYfile
 * (SurfaceReconstruction.cu:58) and DiffuseGeneration's saveDiffuseVTKfile
 * (DiffuseGeneration.cu:847-849) -- and serves the frame from memory
 * (ref_cuda_harness.cu implements them).
 */
#pragma once
#include <cstdint>
#include <vector>
#include "Params.h"
#include "Define.h"
#include "GPUmemory.h"

class FileData {
public:
    int frameIndex = 0;
    FileData(Params* params, GPUmemory* gMemory);
    void loadFluidFile(int frameIndex, float3& motion);
    void saveSurfacePLYfile();
    void saveDiffuseVTKfile(std::vector<DiffuseParticle> diffuse, uint type);

private:
    Params* params;
    GPUmemory* gMemory;
};
