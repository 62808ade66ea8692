// k_mc.cu -- marching cubes over the narrow band.
//
// Reference: MarchingCube_kernel.cuh:20-157 and MarchingCube.cu:32-151.
// detectValidSurfaceCubes: the cube whose origin is band vertex (x,y,z) is
// classified only if all 8 corners are band vertices; its case has bit k set
// when field(corner k) <= iso (corner k at offset {000,001,011,010,100,101,
// 111,110} in (x,y,z), myCuda.cuh:205-257); numVertices[case] mesh vertices
// follow.  Two thrust scans give valid-cube and vertex offsets,
// compactValidSurfaceCubes lists valid cubes, generateTriangles interpolates
// the 12 edge points (getLerpFac, myCuda.cuh:332-339) and normals (central
// differences of the field, zero outside the grid and outside the band,
// myCuda.cuh:259-289) and writes the triangle soup in table order.
//
// GB300 design: the field is read from the dense scalar-grid copy the field
// kernel writes (0 off the band, so a normal's out-of-band neighbour reads 0
// as in the reference); band membership comes from the band bitmap.  One scan
// over packed 64-bit keys (valid << 32 | nvert) yields both offsets; the
// compaction writes one 16-byte record per valid cube {vertex id, case, first
// mesh vertex}, so the emission reads its inputs coalesced.  Each warp emits
// 32 consecutive valid cubes: their mesh vertices are contiguous, so the warp
// stages them in shared memory and writes whole lines (scattered 4-byte stores
// from each cube would leave partial sectors for the memory to merge).  Tables
// sit in constant memory.
#include "pms_internal.h"
#include "k_common.cuh"

namespace pms {

__constant__ uint32_t c_edge_flags[256];
__constant__ int8_t c_tri[256][16];
__constant__ uint8_t c_num_vertices[256];
__constant__ uint8_t c_edge_vertex[12][2];

static constexpr int kThreads = 128;
__device__ __constant__ int c_corner[8][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {0, 1, 0},
                                              {1, 0, 0}, {1, 0, 1}, {1, 1, 1}, {1, 1, 0}};
// c_partner[k][a]: the corner that differs from corner k only along axis a
__device__ __constant__ int c_partner[8][3] = {{4, 3, 1}, {5, 2, 0}, {6, 1, 3}, {7, 0, 2},
                                               {0, 7, 5}, {1, 6, 4}, {2, 5, 7}, {3, 4, 6}};

pms_status upload_mc_tables(pms_ctx* ctx) {
    const McTables& T = mc_tables_host();
    int8_t tri[256][16];
    uint8_t nv[256];
    uint8_t ev[12][2];
    for (int c = 0; c < 256; ++c) {
        nv[c] = (uint8_t)T.num_vertices[c];
        for (int k = 0; k < 16; ++k) tri[c][k] = (int8_t)T.tri[c][k];
    }
    for (int e = 0; e < 12; ++e) { ev[e][0] = (uint8_t)T.edge_vertex[e][0]; ev[e][1] = (uint8_t)T.edge_vertex[e][1]; }
    PMS_CUDA(ctx, cudaMemcpyToSymbol(c_edge_flags, T.edge_flags, sizeof(T.edge_flags)));
    PMS_CUDA(ctx, cudaMemcpyToSymbol(c_tri, tri, sizeof(tri)));
    PMS_CUDA(ctx, cudaMemcpyToSymbol(c_num_vertices, nv, sizeof(nv)));
    PMS_CUDA(ctx, cudaMemcpyToSymbol(c_edge_vertex, ev, sizeof(ev)));
    return PMS_OK;
}

// detectValidSurfaceCubes (6-argument version)
__global__ void __launch_bounds__(kThreads) k_mc_classify(KGrid g, float iso, const Counters* __restrict__ cnt,
                                                          const uint32_t* __restrict__ vlist, const uint32_t* __restrict__ bm,
                                                          const float* __restrict__ fdense, uint32_t* __restrict__ mc_case,
                                                          unsigned long long* __restrict__ mc_key) {
    const uint32_t nv = cnt->nv;
    const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
    const uint64_t nbits = g.sc_size;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nv; t += gridDim.x * blockDim.x) {
        const uint32_t id = vlist[t];
        const uint32_t z = id / rxy, rem = id - z * rxy, y = rem / rx, x = rem - y * rx;
        uint32_t cs = 0, nvert = 0;
        bool all = true;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            // uint32 corner index as getCornerIndex1Ds computes it
            const uint32_t cid = (z + c_corner[k][2]) * rxy + (y + c_corner[k][1]) * rx + (x + c_corner[k][0]);
            const bool in = bit_get(bm, nbits, cid);
            all = all && in;
            if (in) cs |= (__ldg(&fdense[cid]) <= iso ? 1u : 0u) << k;
        }
        if (all) nvert = c_num_vertices[cs];
        else cs = 0;
        mc_case[t] = cs;
        mc_key[t] = nvert ? ((1ull << 32) | nvert) : 0ull;
    }
}

// unpack the scanned total {valid cubes << 32 | mesh vertices} into the counters
__global__ void k_mc_totals(const unsigned long long* __restrict__ total, Counters* __restrict__ cnt) {
    const unsigned long long t = *total;
    cnt->nvalid = (uint32_t)(t >> 32);
    cnt->nmesh = t & 0xffffffffull;
}

// compactValidSurfaceCubes, plus the emission's per-cube record
__global__ void __launch_bounds__(256) k_mc_compact(const Counters* __restrict__ cnt,
                                                    const unsigned long long* __restrict__ mc_key,
                                                    const unsigned long long* __restrict__ mc_off,
                                                    const uint32_t* __restrict__ vlist, const uint32_t* __restrict__ mc_case,
                                                    uint32_t* __restrict__ valid, uint4* __restrict__ cube) {
    const uint32_t nv = cnt->nv;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nv; t += gridDim.x * blockDim.x)
        if (mc_key[t]) {
            const unsigned long long off = mc_off[t];
            const uint32_t k = (uint32_t)(off >> 32);
            valid[k] = t;
            cube[k] = make_uint4(vlist[t], mc_case[t], (uint32_t)(off & 0xffffffffull), 0u);
        }
}

// field at scalar-grid vertex (x, y, z): 0 outside the grid and off the band
__device__ __forceinline__ float grid_value(const KGrid& g, const float* __restrict__ fdense, int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0 || (uint32_t)x >= g.scres[0] || (uint32_t)y >= g.scres[1] || (uint32_t)z >= g.scres[2])
        return 0.f;
    return __ldg(&fdense[((size_t)z * g.scres[1] + (size_t)y) * g.scres[0] + (size_t)x]);
}

__device__ __forceinline__ float3 normalized(float3 v) {
    const float inv = 1.f / sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    return make_float3(v.x * inv, v.y * inv, v.z * inv);
}

// generateTriangles: one thread per valid cube, a warp per 32 consecutive cubes
static constexpr int kEmitWarps = kThreads / 32;
static constexpr int kEmitStage = 32 * 15 * 3;     // floats: 32 cubes x 15 mesh vertices x 3

__global__ void __launch_bounds__(kThreads) k_mc_emit(KGrid g, float iso, Counters* __restrict__ cnt,
                                                      const uint4* __restrict__ cube, const float* __restrict__ fdense,
                                                      float* __restrict__ vert, float* __restrict__ vnorm,
                                                      const unsigned long long* __restrict__ frame_base,
                                                      unsigned long long cap) {
    __shared__ float stage[kEmitWarps][kEmitStage];
    const uint32_t nvalid = cnt->nvalid;
    // batched frames write behind the earlier frames' vertices, within cap
    const unsigned long long fb = frame_base ? *frame_base : 0ull;
    const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
    const float sgn = (iso < 0.f) ? -1.f : 1.f;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* st = stage[warp];
    for (uint32_t k0 = (blockIdx.x * kEmitWarps + warp) * 32u; k0 < nvalid; k0 += gridDim.x * kEmitWarps * 32u) {
        const uint32_t k = k0 + (uint32_t)lane;
        const bool active = k < nvalid;
        const uint4 cr = active ? __ldg(&cube[k]) : make_uint4(0u, 0u, 0u, 0u);
        const uint32_t id = cr.x, cs = cr.y, base = cr.z;
        const uint32_t nvert = active ? (uint32_t)c_num_vertices[cs] : 0u;
        // the warp's mesh vertices are [base0, base0 + total)
        const int last = (int)min(31u, nvalid - 1u - k0);
        const uint32_t base0 = __shfl_sync(0xffffffffu, base, 0);
        const uint32_t total = __shfl_sync(0xffffffffu, base + nvert, last) - base0;
        const unsigned long long w0 = fb + base0;
        const uint32_t room = w0 >= cap ? 0u : (cap - w0 < (unsigned long long)total ? (uint32_t)(cap - w0) : total);
        if (room < total && lane == 0) atomicOr(&cnt->err, kErrCapacity);
        float3 ip[12], in[12];
        if (nvert) {
            const int z = (int)(id / rxy), rem = (int)(id - (uint32_t)z * rxy), y = rem / (int)rx, x = rem - y * (int)rx;
            float3 cp[8], cn[8];
            float cf[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int X = x + c_corner[c][0], Y = y + c_corner[c][1], Z = z + c_corner[c][2];
                cp[c] = make_float3(sc_coord_i(g, X, 0), sc_coord_i(g, Y, 1), sc_coord_i(g, Z, 2));
                cf[c] = __ldg(&fdense[(size_t)Z * rxy + (size_t)Y * rx + (size_t)X]);   // a band vertex
            }
            // central differences (getVertexNorm): along each axis one neighbour of a corner
            // is the cube's other corner on that axis, the other lies outside the cube
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int ox = c_corner[c][0], oy = c_corner[c][1], oz = c_corner[c][2];
                const int X = x + ox, Y = y + oy, Z = z + oz;
                const float fx = grid_value(g, fdense, ox ? X + 1 : X - 1, Y, Z);
                const float fy = grid_value(g, fdense, X, oy ? Y + 1 : Y - 1, Z);
                const float fz = grid_value(g, fdense, X, Y, oz ? Z + 1 : Z - 1);
                const float px = cf[c_partner[c][0]], py = cf[c_partner[c][1]], pz = cf[c_partner[c][2]];
                float3 n;
                n.x = ox ? px - fx : fx - px;
                n.y = oy ? py - fy : fy - py;
                n.z = oz ? pz - fz : fz - pz;
                cn[c] = normalized(n);
            }
            const uint32_t ef = c_edge_flags[cs];
#pragma unroll
            for (int e = 0; e < 12; ++e) {
                if (!(ef & (1u << e))) continue;
                const int a = c_edge_vertex[e][0], b = c_edge_vertex[e][1];
                const float d = cf[b] - cf[a];
                // getLerpFac: |delta| < 1e-7 (a double literal) -> 0.5
                const float tt = ((double)d > -1.0e-7 && (double)d < 1.0e-7) ? 0.5f : (iso - cf[a]) / d;
                ip[e] = make_float3(cp[a].x + tt * (cp[b].x - cp[a].x), cp[a].y + tt * (cp[b].y - cp[a].y),
                                    cp[a].z + tt * (cp[b].z - cp[a].z));
                const float3 nn = normalized(make_float3(cn[a].x + tt * (cn[b].x - cn[a].x),
                                                         cn[a].y + tt * (cn[b].y - cn[a].y),
                                                         cn[a].z + tt * (cn[b].z - cn[a].z)));
                in[e] = make_float3(sgn * nn.x, sgn * nn.y, sgn * nn.z);
            }
        }
        // positions, then normals: stage the warp's vertices in order, write whole lines
        const uint32_t o = base - base0;
        for (uint32_t v = 0; v < nvert; ++v) {
            const float3 p = ip[c_tri[cs][v]];
            st[3 * (o + v)] = p.x; st[3 * (o + v) + 1] = p.y; st[3 * (o + v) + 2] = p.z;
        }
        __syncwarp();
        for (uint32_t i = (uint32_t)lane; i < 3u * room; i += 32u) vert[3 * (size_t)w0 + i] = st[i];
        __syncwarp();
        if (vnorm) {
            for (uint32_t v = 0; v < nvert; ++v) {
                const float3 q = in[c_tri[cs][v]];
                st[3 * (o + v)] = q.x; st[3 * (o + v) + 1] = q.y; st[3 * (o + v) + 2] = q.z;
            }
            __syncwarp();
            for (uint32_t i = (uint32_t)lane; i < 3u * room; i += 32u) vnorm[3 * (size_t)w0 + i] = st[i];
            __syncwarp();
        }
    }
}

pms_status launch_mc_classify(pms_ctx* ctx) {
    const KGrid g = kgrid_of(ctx->grid);
    Counters* cnt = ctx->counters.as<Counters>();
    k_mc_classify<<<grid_for(ctx->nv, kThreads), kThreads, 0, ctx->stream>>>(
        g, ctx->prm.iso_value, cnt, ctx->vlist.as<uint32_t>(), ctx->bm.as<uint32_t>(), ctx->fdense.as<float>(),
        ctx->mc_case.as<uint32_t>(), ctx->mc_key.as<unsigned long long>());
    PMS_LAUNCHED(ctx);
    // ctx->nv may be a bound (batched frames): the scan stops at the device count
    pms_status st = scan_u64(ctx, ctx->mc_key.as<unsigned long long>(), ctx->mc_off.as<unsigned long long>(), ctx->nv,
                             ctx->tmp.as<unsigned long long>(), &cnt->nv);
    if (st != PMS_OK) return st;
    k_mc_totals<<<1, 1, 0, ctx->stream>>>(ctx->tmp.as<unsigned long long>(), cnt);
    PMS_LAUNCHED(ctx);
    k_mc_compact<<<grid_for(ctx->nv, 256), 256, 0, ctx->stream>>>(
        cnt, ctx->mc_key.as<unsigned long long>(), ctx->mc_off.as<unsigned long long>(), ctx->vlist.as<uint32_t>(),
        ctx->mc_case.as<uint32_t>(), ctx->valid.as<uint32_t>(), ctx->cube.as<uint4>());
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

// ---------------------------------------------------------------------------
// estimationOfScalarValue (MarchingCube_kernel.cuh:161-233, called after the
// triangles by MarchingCube::triangulation, MarchingCube.cu:50-52): density
// and velocity at every mesh vertex, averaged over the particles within h of
// it with w = 1 - (d/h)^3, over the cells [c - e, c + e) of the vertex's
// spatial cell (upper bound exclusive, as the reference).  Out: 5 floats per
// vertex {vel xyz, |vel|, rhop}, the reference's ScalarValue; zero where no
// particle is within h.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_scalar_values(KGrid g, float h, const Counters* __restrict__ cnt,
                                                            const float* __restrict__ vert,
                                                            const uint32_t* __restrict__ cell_start,
                                                            const float4* __restrict__ spos, const float4* __restrict__ svel,
                                                            const float* __restrict__ rho, float* __restrict__ out) {
    const unsigned long long m = cnt->nmesh;
    const float pad = 1e-4f * g.sp_cs;
    for (unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; t < m;
         t += (unsigned long long)gridDim.x * blockDim.x) {
        const float3 v = make_float3(vert[3 * t], vert[3 * t + 1], vert[3 * t + 2]);
        const uint3 c = sp_cell(g, v.x, v.y, v.z);
        uint3 lo, hi;
        box_clamp(g, c, (uint32_t)g.spexpand, lo, hi);   // loops run to hi exclusive, as the reference's
        float ws = 0.f, rh = 0.f, vx = 0.f, vy = 0.f, vz = 0.f;
        row_walk(g, v, lo, hi, h * h, pad, cell_start, [&](uint32_t j) {
            const float4 q = __ldg(&spos[j]);
            const float dx = v.x - q.x, dy = v.y - q.y, dz = v.z - q.z;
            const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
            if (dist < h) {
                const float s = dist / h;
                const float w = 1.f - s * s * s;
                const float4 u = __ldg(&svel[j]);
                rh += w * __ldg(&rho[j]);
                vx += w * u.x; vy += w * u.y; vz += w * u.z;
                ws += w;
            }
        });
        float* o = out + 5 * t;
        if (ws > 0.f) {
            rh /= ws; vx /= ws; vy /= ws; vz /= ws;
            o[0] = vx; o[1] = vy; o[2] = vz; o[3] = sqrtf(vx * vx + vy * vy + vz * vz); o[4] = rh;
        } else {
            o[0] = o[1] = o[2] = o[3] = o[4] = 0.f;
        }
    }
}

pms_status launch_scalar_values(pms_ctx* ctx) {
    const KGrid g = kgrid_of(ctx->grid);
    k_scalar_values<<<grid_for(ctx->nmesh, kThreads), kThreads, 0, ctx->stream>>>(
        g, ctx->prm.h, ctx->counters.as<Counters>(), ctx->vert.as<float>(), ctx->cell_start.as<uint32_t>(),
        ctx->spos.as<float4>(), ctx->svel.as<float4>(), ctx->rho.as<float>(), ctx->sval.as<float>());
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

// batched frames: this frame's mesh takes the next free stretch of the arena
// (frames of different lanes run concurrently, so the claim is atomic)
__global__ void k_batch_base(const Counters* __restrict__ cnt, unsigned long long* __restrict__ running,
                             unsigned long long* __restrict__ base) {
    *base = atomicAdd(running, (unsigned long long)cnt->nmesh);
}

pms_status launch_batch_base(pms_ctx* ctx, const Counters* cnt, unsigned long long* running, unsigned long long* base) {
    k_batch_base<<<1, 1, 0, ctx->stream>>>(cnt, running, base);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_mc_emit_to(pms_ctx* ctx, float* vert, float* vnorm, const unsigned long long* frame_base,
                             unsigned long long cap) {
    const KGrid g = kgrid_of(ctx->grid);
    Counters* cnt = ctx->counters.as<Counters>();
    k_mc_emit<<<grid_for(ctx->nvalid, kThreads), kThreads, 0, ctx->stream>>>(
        g, ctx->prm.iso_value, cnt, ctx->cube.as<uint4>(), ctx->fdense.as<float>(), vert, vnorm, frame_base, cap);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_mc_emit(pms_ctx* ctx) {
    return launch_mc_emit_to(ctx, ctx->vert.as<float>(), ctx->vnorm.as<float>(), nullptr, ~0ull);
}

}  // namespace pms
