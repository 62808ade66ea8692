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

// Case tables in global memory: lanes of a warp look up different cases, which
// constant memory would serialise.  g_case[c] = edge flags (bits 0-11) | number
// of mesh vertices << 16; g_slots[c][e] = the mesh vertices (bit v) of case c
// that lie on edge e.
__device__ uint32_t g_case[256];
__device__ uint16_t g_slots[256][12];

static constexpr int kThreads = 128;

// Corner c's offset along axis a, for the corner order {000, 001, 011, 010,
// 100, 101, 111, 110} in (x, y, z) (myCuda.cuh:205-216); the corner that
// differs from c only along axis a; the end corners of edge e
// (vertexIndexesOfEdge: the four edges of the x = 0 face, of the x = 1 face,
// then the four along x).  The emission is compiled for this edge numbering
// and the table upload checks that the active tables use it.
__host__ __device__ constexpr int corner_off(int c, int a) {
    return a == 0 ? (c >> 2) : a == 1 ? ((c >> 1) & 1) : ((c & 1) ^ ((c >> 1) & 1));
}
__host__ __device__ constexpr int corner_at(int x, int y, int z) { return 4 * x + 2 * y + (y ^ z); }
__host__ __device__ constexpr int corner_partner(int c, int a) {
    return corner_at(corner_off(c, 0) ^ (a == 0), corner_off(c, 1) ^ (a == 1), corner_off(c, 2) ^ (a == 2));
}
__host__ __device__ constexpr int edge_end(int e, int i) {
    return e < 8 ? (i == 0 ? e : (e & 4) + ((e + 1) & 3)) : (i == 0 ? e - 8 : e - 4);
}

pms_status upload_mc_tables(pms_ctx* ctx) {
    const McTables& T = mc_tables_host();
    for (int e = 0; e < 12; ++e)
        if ((int)T.edge_vertex[e][0] != edge_end(e, 0) || (int)T.edge_vertex[e][1] != edge_end(e, 1))
            return pms_fail(ctx, PMS_ERR_UNSUPPORTED, "marching-cubes tables number the cube edges differently");
    uint32_t cs[256];
    uint16_t slots[256][12];
    for (int c = 0; c < 256; ++c) {
        cs[c] = (T.edge_flags[c] & 0xfffu) | (T.num_vertices[c] << 16);
        for (int e = 0; e < 12; ++e) slots[c][e] = 0;
        for (uint32_t v = 0; v < T.num_vertices[c] && v < 16; ++v) {
            const int e = T.tri[c][v];
            if (e < 0 || e >= 12) return pms_fail(ctx, PMS_ERR_UNSUPPORTED, "marching-cubes table: edge %d in case %d", e, c);
            slots[c][e] |= (uint16_t)(1u << v);
        }
    }
    PMS_CUDA(ctx, cudaMemcpyToSymbol(g_case, cs, sizeof(cs)));
    PMS_CUDA(ctx, cudaMemcpyToSymbol(g_slots, slots, sizeof(slots)));
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
            const uint32_t cid = (z + corner_off(k, 2)) * rxy + (y + corner_off(k, 1)) * rx + (x + corner_off(k, 0));
            const bool in = bit_get(bm, nbits, cid);
            all = all && in;
            if (in) cs |= (__ldg(&fdense[cid]) <= iso ? 1u : 0u) << k;
        }
        if (all) nvert = __ldg(&g_case[cs]) >> 16;
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

// generateTriangles: one thread per valid cube, a warp per 32 consecutive cubes.
// Every edge's point and normal go straight to the mesh vertices of the case
// that use it (g_slots), staged per warp as {position, normal}.
static constexpr int kEmitWarps = kThreads / 32;
static constexpr int kEmitStage = 32 * 15 * 6;     // floats: 32 cubes x 15 mesh vertices x {p, n}

// kNormals: also the vertex normals (into vnorm); without them only positions
// are made, from the same arithmetic, so the positions are the same either way.
template <bool kNormals>
__global__ void __launch_bounds__(kThreads) k_mc_emit(KGrid g, float iso, Counters* __restrict__ cnt,
                                                      const uint4* __restrict__ cube, const float* __restrict__ fdense,
                                                      float* __restrict__ vert, float* __restrict__ vnorm,
                                                      const unsigned long long* __restrict__ frame_base,
                                                      unsigned long long cap, int piece) {
    constexpr int kS = kNormals ? 6 : 3;       // staged floats per mesh vertex
    __shared__ float stage[kEmitWarps][kEmitStage / 6 * kS];
    // one streamed piece covers the cubes [mc_piece[piece], mc_piece[piece + 1]); piece < 0: all of them
    const uint32_t ka = piece < 0 ? 0u : cnt->mc_piece[piece];
    const uint32_t nvalid = piece < 0 ? cnt->nvalid : cnt->mc_piece[piece + 1];
    // batched frames write behind the earlier frames' vertices, within cap
    const unsigned long long fb = frame_base ? *frame_base : 0ull;
    const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
    const float sgn = (iso < 0.f) ? -1.f : 1.f;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* st = stage[warp];
    for (uint32_t k0 = ka + (blockIdx.x * kEmitWarps + warp) * 32u; k0 < nvalid; k0 += gridDim.x * kEmitWarps * 32u) {
        const uint32_t k = k0 + (uint32_t)lane;
        const bool active = k < nvalid;
        const uint4 cr = active ? __ldg(&cube[k]) : make_uint4(0u, 0u, 0u, 0u);
        const uint32_t id = cr.x, cs = cr.y, base = cr.z;
        const uint32_t info = __ldg(&g_case[cs]);
        const uint32_t nvert = active ? info >> 16 : 0u, ef = active ? info & 0xfffu : 0u;
        // the warp's mesh vertices are [base0, base0 + total)
        const int last = (int)min(31u, nvalid - 1u - k0);
        const uint32_t base0 = __shfl_sync(0xffffffffu, base, 0);
        const uint32_t total = __shfl_sync(0xffffffffu, base + nvert, last) - base0;
        const unsigned long long w0 = fb + base0;
        const uint32_t room = w0 >= cap ? 0u : (cap - w0 < (unsigned long long)total ? (uint32_t)(cap - w0) : total);
        if (room < total && lane == 0) atomicOr(&cnt->err, kErrCapacity);
        if (nvert) {
            const int z = (int)(id / rxy), rem = (int)(id - (uint32_t)z * rxy), y = rem / (int)rx, x = rem - y * (int)rx;
            // corner coordinates: axis value of offset 0 and 1
            const float px[2] = {sc_coord_i(g, x, 0), sc_coord_i(g, x + 1, 0)};
            const float py[2] = {sc_coord_i(g, y, 1), sc_coord_i(g, y + 1, 1)};
            const float pz[2] = {sc_coord_i(g, z, 2), sc_coord_i(g, z + 1, 2)};
            float cf[8];
#pragma unroll
            for (int c = 0; c < 8; ++c)    // band vertices: the uint32 index the classification used
                cf[c] = __ldg(&fdense[(uint32_t)(z + corner_off(c, 2)) * rxy + (uint32_t)(y + corner_off(c, 1)) * rx +
                                      (uint32_t)(x + corner_off(c, 0))]);
            // central differences (getVertexNorm): along each axis one neighbour of a corner
            // is the cube's other corner on that axis, the other lies outside the cube
            float3 cn[8];
#pragma unroll
            for (int c = 0; c < 8 && kNormals; ++c) {
                const int ox = corner_off(c, 0), oy = corner_off(c, 1), oz = corner_off(c, 2);
                const int X = x + ox, Y = y + oy, Z = z + oz;
                const float fx = grid_value(g, fdense, ox ? X + 1 : X - 1, Y, Z);
                const float fy = grid_value(g, fdense, X, oy ? Y + 1 : Y - 1, Z);
                const float fz = grid_value(g, fdense, X, Y, oz ? Z + 1 : Z - 1);
                const float qx = cf[corner_partner(c, 0)], qy = cf[corner_partner(c, 1)], qz = cf[corner_partner(c, 2)];
                cn[c] = normalized(make_float3(ox ? qx - fx : fx - qx, oy ? qy - fy : fy - qy, oz ? qz - fz : fz - qz));
            }
            const uint32_t o = base - base0;
            const uint16_t* slots = g_slots[cs];
#pragma unroll
            for (int e = 0; e < 12; ++e) {
                if (!(ef & (1u << e))) continue;
                const int a = edge_end(e, 0), b = edge_end(e, 1);
                const float d = cf[b] - cf[a];
                // getLerpFac: |delta| < 1e-7 (a double literal) -> 0.5.  1e-7f, the float
                // nearest 1e-7, lies above it and no float lies between them, so for a float
                // delta the double test is |delta| < 1e-7f: the same decision without the
                // FP64 pipe
                const float tt = fabsf(d) < 1.0e-7f ? 0.5f : (iso - cf[a]) / d;
                const float ax = px[corner_off(a, 0)], ay = py[corner_off(a, 1)], az = pz[corner_off(a, 2)];
                const float bx = px[corner_off(b, 0)], by = py[corner_off(b, 1)], bz = pz[corner_off(b, 2)];
                float q[kS];
                q[0] = ax + tt * (bx - ax);
                q[1] = ay + tt * (by - ay);
                q[2] = az + tt * (bz - az);
                if constexpr (kNormals) {
                    const float3 nn = normalized(make_float3(cn[a].x + tt * (cn[b].x - cn[a].x),
                                                             cn[a].y + tt * (cn[b].y - cn[a].y),
                                                             cn[a].z + tt * (cn[b].z - cn[a].z)));
                    q[3] = sgn * nn.x;
                    q[4] = sgn * nn.y;
                    q[5] = sgn * nn.z;
                }
                for (uint32_t m = __ldg(&slots[e]); m; m &= m - 1u) {
                    float* dst = st + kS * (o + (uint32_t)(__ffs(m) - 1));
#pragma unroll
                    for (int c = 0; c < kS; ++c) dst[c] = q[c];
                }
            }
        }
        __syncwarp();
        // whole lines: positions, then normals
        if constexpr (kNormals) {
            for (uint32_t i = (uint32_t)lane; i < 3u * room; i += 32u) {
                const uint32_t v = i / 3u, c = i - 3u * v;
                vert[3 * (size_t)w0 + i] = st[6 * v + c];
            }
            for (uint32_t i = (uint32_t)lane; i < 3u * room; i += 32u) {
                const uint32_t v = i / 3u, c = i - 3u * v;
                vnorm[3 * (size_t)w0 + i] = st[6 * v + 3 + c];
            }
        } else {
            for (uint32_t i = (uint32_t)lane; i < 3u * room; i += 32u) vert[3 * (size_t)w0 + i] = st[i];
        }
        __syncwarp();
    }
}

pms_status launch_mc_cases(pms_ctx* ctx) {
    const KGrid g = kgrid_of(ctx->grid);
    Counters* cnt = ctx->counters.as<Counters>();
    k_mc_classify<<<grid_for(ctx->nv, kThreads), kThreads, 0, ctx->stream>>>(
        g, ctx->prm.iso_value, cnt, ctx->vlist.as<uint32_t>(), ctx->bm.as<uint32_t>(), ctx->fdense.as<float>(),
        ctx->mc_case.as<uint32_t>(), ctx->mc_key.as<unsigned long long>());
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_mc_compact(pms_ctx* ctx) {
    Counters* cnt = ctx->counters.as<Counters>();
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

pms_status launch_mc_classify(pms_ctx* ctx) {
    pms_status st = launch_mc_cases(ctx);
    return st ? st : launch_mc_compact(ctx);
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

// A batched frame's triangle soup into mapped page-locked host memory, at the same
// vertex offset as in the device arena: stores over the host link from the SMs, on
// the frame's lane right after its emission, while the other lanes compute.  What
// lies past the host arena's capacity is left out and flagged in *trunc.
__global__ void __launch_bounds__(256) k_batch_mesh_to_host(const float* __restrict__ mesh,
                                                            const unsigned long long* __restrict__ base_f,
                                                            const Counters* __restrict__ cnt, unsigned long long dev_cap,
                                                            float* __restrict__ host, unsigned long long host_cap,
                                                            uint32_t* __restrict__ trunc) {
    const unsigned long long b = *base_f;
    unsigned long long n = cnt->nmesh;
    if (b >= dev_cap) return;                          // the device arena overflowed: the batch runs again
    if (b + n > dev_cap) n = dev_cap - b;
    if (b + n > host_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(trunc, 1u);
        n = b < host_cap ? host_cap - b : 0ull;
    }
    const float* __restrict__ src = mesh + 3 * b;
    float* __restrict__ dst = host + 3 * b;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < 3 * n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        dst[i] = __ldcs(src + i);
}

pms_status launch_batch_mesh_to_host(pms_ctx* ctx, const float* mesh, const unsigned long long* base_f,
                                     unsigned long long dev_cap, float* host, unsigned long long host_cap, uint32_t* trunc) {
    k_batch_mesh_to_host<<<152 * 2, 256, 0, ctx->stream>>>(mesh, base_f, ctx->counters.as<Counters>(), dev_cap, host,
                                                          host_cap, trunc);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_batch_base(pms_ctx* ctx, const Counters* cnt, unsigned long long* running, unsigned long long* base) {
    k_batch_base<<<1, 1, 0, ctx->stream>>>(cnt, running, base);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

// The first cube of each of `pieces` vertex ranges: cube records are in ascending
// first-vertex order, so it is the lower bound of the range's first vertex.
__global__ void k_mc_piece_bounds(const uint4* __restrict__ cube, Counters* __restrict__ cnt, uint32_t pieces) {
    const uint32_t q = threadIdx.x;
    if (q > pieces) return;
    const uint32_t n = cnt->nvalid;
    uint32_t lo = 0u, hi = n;
    if (q == pieces) lo = n;
    else if (q > 0u) {
        const uint32_t v = (uint32_t)(cnt->nmesh * q / pieces);
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (cube[mid].z < v) lo = mid + 1u;
            else hi = mid;
        }
    }
    cnt->mc_piece[q] = lo;
}

pms_status launch_mc_piece_bounds(pms_ctx* ctx, uint32_t pieces) {
    if (pieces < 1u || pieces > (uint32_t)kMaxMcPieces) return pms_fail(ctx, PMS_ERR_INVALID_ARGUMENT, "emission pieces");
    k_mc_piece_bounds<<<1, 32, 0, ctx->stream>>>(ctx->cube.as<uint4>(), ctx->counters.as<Counters>(), pieces);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_mc_emit_to(pms_ctx* ctx, float* vert, float* vnorm, const unsigned long long* frame_base,
                             unsigned long long cap, int piece, uint32_t pieces) {
    const KGrid g = kgrid_of(ctx->grid);
    Counters* cnt = ctx->counters.as<Counters>();
    // a piece's grid covers its share of the cubes with room for an uneven split; the
    // grid-stride loop takes whatever is left over
    const uint64_t work = piece < 0 ? ctx->nvalid : ((uint64_t)ctx->nvalid * 5u / (4u * pieces) + 1u);
    const unsigned blocks = grid_for(work, kThreads);
    if (vnorm)
        k_mc_emit<true><<<blocks, kThreads, 0, ctx->stream>>>(g, ctx->prm.iso_value, cnt, ctx->cube.as<uint4>(),
                                                              ctx->fdense.as<float>(), vert, vnorm, frame_base, cap,
                                                              piece);
    else
        k_mc_emit<false><<<blocks, kThreads, 0, ctx->stream>>>(g, ctx->prm.iso_value, cnt, ctx->cube.as<uint4>(),
                                                               ctx->fdense.as<float>(), vert, nullptr, frame_base,
                                                               cap, piece);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

// ---------------------------------------------------------------------------
// Welded mesh (no counterpart in the reference, whose PLY and VTK surface files
// hold the triangle soup, FileData.cpp:677-773 and 1277-1332).  Neighbouring
// cubes share their crossed grid edges; the welded mesh keeps one vertex per
// crossed edge and a triangle index list in the soup's order.  A grid edge is
// keyed by its lower corner and its axis, 3 * vertex id + axis.  Its point is
// interpolated once, from the lower to the upper corner; the soup interpolates
// it in every cube that uses it, from whichever end that cube's table names
// first, so the two agree up to the rounding of that choice.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t edge_key(uint32_t id, uint32_t rx, uint32_t rxy, int e) {
    const int a = edge_end(e, 0), b = edge_end(e, 1);
    const int axis = corner_off(a, 0) != corner_off(b, 0) ? 0 : (corner_off(a, 1) != corner_off(b, 1) ? 1 : 2);
    const int lo = corner_off(a, axis) < corner_off(b, axis) ? a : b;
    const uint32_t v = id + (uint32_t)corner_off(lo, 0) + (uint32_t)corner_off(lo, 1) * rx + (uint32_t)corner_off(lo, 2) * rxy;
    return 3ull * v + (uint64_t)axis;
}

__global__ void __launch_bounds__(256) k_weld_mark(KGrid g, const Counters* __restrict__ cnt, const uint4* __restrict__ cube,
                                                   uint32_t* __restrict__ ebits) {
    const uint32_t n = cnt->nvalid;
    const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint4 cr = __ldg(&cube[t]);
        const uint32_t ef = __ldg(&g_case[cr.y]) & 0xfffu;
        for (uint32_t m = ef; m; m &= m - 1u) {
            const uint64_t key = edge_key(cr.x, rx, rxy, __ffs(m) - 1);
            const uint32_t bit = 1u << (key & 31u);
            if (!(ebits[key >> 5] & bit)) atomicOr(&ebits[key >> 5], bit);
        }
    }
}

__global__ void __launch_bounds__(256) k_weld_popc(const uint32_t* __restrict__ b, uint32_t* __restrict__ wc, uint64_t nw) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nw; w += (uint64_t)gridDim.x * blockDim.x)
        wc[w] = __popc(b[w]);
}

// the negative field gradient at a scalar vertex (central differences, 0 outside the grid
// and the band), the vertex normal of getVertexNorm (myCuda.cuh:259-289)
__device__ __forceinline__ float3 vertex_normal(const KGrid& g, const float* __restrict__ fdense, int x, int y, int z) {
    return normalized(make_float3(grid_value(g, fdense, x - 1, y, z) - grid_value(g, fdense, x + 1, y, z),
                                  grid_value(g, fdense, x, y - 1, z) - grid_value(g, fdense, x, y + 1, z),
                                  grid_value(g, fdense, x, y, z - 1) - grid_value(g, fdense, x, y, z + 1)));
}

// one welded vertex per set edge bit, at the edge's rank
__global__ void __launch_bounds__(256) k_weld_vertices(KGrid g, float iso, const uint32_t* __restrict__ ebits,
                                                       const uint32_t* __restrict__ wprefix, uint64_t nw,
                                                       const float* __restrict__ fdense, uint64_t cap,
                                                       float* __restrict__ vert, float* __restrict__ vnorm) {
    const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
    const float sgn = (iso < 0.f) ? -1.f : 1.f;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nw; w += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t bits = ebits[w], r = wprefix[w];
        while (bits) {
            const uint32_t bi = (uint32_t)(__ffs(bits) - 1);
            bits &= bits - 1u;
            if (r >= cap) break;   // the host sizes vert for every soup vertex; never reached
            const uint64_t key = 32ull * w + bi;
            const uint32_t v = (uint32_t)(key / 3ull), axis = (uint32_t)(key - 3ull * v);
            const int z = (int)(v / rxy), rem = (int)(v - (uint32_t)z * rxy), y = rem / (int)rx, x = rem - y * (int)rx;
            const int X = x + (axis == 0), Y = y + (axis == 1), Z = z + (axis == 2);
            const float fa = grid_value(g, fdense, x, y, z), fb = grid_value(g, fdense, X, Y, Z);
            const float d = fb - fa;
            const float tt = fabsf(d) < 1.0e-7f ? 0.5f : (iso - fa) / d;   // getLerpFac's test, as above
            const float ax = sc_coord_i(g, x, 0), ay = sc_coord_i(g, y, 1), az = sc_coord_i(g, z, 2);
            const float bx = sc_coord_i(g, X, 0), by = sc_coord_i(g, Y, 1), bz = sc_coord_i(g, Z, 2);
            vert[3 * (size_t)r + 0] = ax + tt * (bx - ax);
            vert[3 * (size_t)r + 1] = ay + tt * (by - ay);
            vert[3 * (size_t)r + 2] = az + tt * (bz - az);
            if (vnorm) {
                const float3 na = vertex_normal(g, fdense, x, y, z), nb = vertex_normal(g, fdense, X, Y, Z);
                const float3 nn = normalized(make_float3(na.x + tt * (nb.x - na.x), na.y + tt * (nb.y - na.y),
                                                         na.z + tt * (nb.z - na.z)));
                vnorm[3 * (size_t)r + 0] = sgn * nn.x;
                vnorm[3 * (size_t)r + 1] = sgn * nn.y;
                vnorm[3 * (size_t)r + 2] = sgn * nn.z;
            }
            ++r;
        }
    }
}

// the triangle index list, in the soup's order: mesh vertex base + slot of a valid cube
// takes the rank of the edge its table entry names
__global__ void __launch_bounds__(256) k_weld_indices(KGrid g, const Counters* __restrict__ cnt, const uint4* __restrict__ cube,
                                                      const uint32_t* __restrict__ ebits, const uint32_t* __restrict__ wprefix,
                                                      uint32_t* __restrict__ idx) {
    const uint32_t n = cnt->nvalid;
    const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint4 cr = __ldg(&cube[t]);
        const uint32_t ef = __ldg(&g_case[cr.y]) & 0xfffu;
        for (uint32_t m = ef; m; m &= m - 1u) {
            const int e = __ffs(m) - 1;
            const uint64_t key = edge_key(cr.x, rx, rxy, e);
            const uint32_t w = (uint32_t)(key >> 5), bi = (uint32_t)(key & 31u);
            const uint32_t rank = wprefix[w] + __popc(ebits[w] & ((1u << bi) - 1u));
            for (uint32_t sl = __ldg(&g_slots[cr.y][e]); sl; sl &= sl - 1u)
                idx[(size_t)cr.z + (uint32_t)(__ffs(sl) - 1)] = rank;
        }
    }
}

pms_status launch_weld(pms_ctx* ctx, uint32_t* ebits, uint32_t* wc, uint32_t* wprefix, uint64_t nw, uint32_t* n_unique,
                       uint64_t cap, float* vert, float* vnorm, uint32_t* idx) {
    const KGrid g = kgrid_of(ctx->grid);
    Counters* cnt = ctx->counters.as<Counters>();
    PMS_CUDA(ctx, cudaMemsetAsync(ebits, 0, 4 * nw, ctx->stream));
    k_weld_mark<<<grid_for(ctx->nvalid, 256), 256, 0, ctx->stream>>>(g, cnt, ctx->cube.as<uint4>(), ebits);
    PMS_LAUNCHED(ctx);
    k_weld_popc<<<grid_for(nw, 256), 256, 0, ctx->stream>>>(ebits, wc, nw);
    PMS_LAUNCHED(ctx);
    pms_status st = scan_u32(ctx, wc, wprefix, nw, n_unique);
    if (st) return st;
    if (vert) {
        k_weld_vertices<<<grid_for(nw, 256), 256, 0, ctx->stream>>>(g, ctx->prm.iso_value, ebits, wprefix, nw,
                                                                    ctx->fdense.as<float>(), cap, vert, vnorm);
        PMS_LAUNCHED(ctx);
    }
    if (idx) {
        k_weld_indices<<<grid_for(ctx->nvalid, 256), 256, 0, ctx->stream>>>(g, cnt, ctx->cube.as<uint4>(), ebits, wprefix, idx);
        PMS_LAUNCHED(ctx);
    }
    return PMS_OK;
}

pms_status launch_mc_emit(pms_ctx* ctx, int piece, uint32_t pieces) {
    return launch_mc_emit_to(ctx, ctx->vert.as<float>(), ctx->mesh_normals ? ctx->vnorm.as<float>() : nullptr, nullptr,
                             ~0ull, piece, pieces);
}

}  // namespace pms
