// k_order.cu -- processing orders with 3D locality for the neighbour walks.
//
// Band vertices are listed in linear (z, y, x) order and particles in cell-key
// order, so consecutive threads spread along x rows and a block's neighbour
// data (positions, kernels, cell records) is spread over a long thin slab
// that does not stay in L1.  These counting sorts produce permutations that
// visit the items tile by tile -- 8 x 8 x 8 scalar vertices, or 4 x 4 x 4
// spatial cells -- so the threads of a block work on one compact region and
// its neighbours are read from L1 rather than L2.  Each item's result is
// written to its own slot, so the order changes no value.
#include "pms_internal.h"
#include "k_common.cuh"

namespace pms {

// tile of band vertex vlist[t]: (x >> 3, y >> 3, z >> 3)
struct VertexTile {
    const uint32_t* vlist;
    uint32_t rx, rxy, tx, ty;
    __device__ uint32_t operator()(uint32_t t) const {
        const uint32_t id = vlist[t];
        const uint32_t z = id / rxy, rem = id - z * rxy, y = rem / rx, x = rem - y * rx;
        return ((z >> 3) * ty + (y >> 3)) * tx + (x >> 3);
    }
};

// tile of particle item i, whose sorted index is idx ? idx[i] : i: spatial cell >> 2
struct ParticleTile {
    const uint32_t* skeys;
    const uint32_t* idx;
    uint32_t sx, sxy, tx, ty;
    __device__ uint32_t operator()(uint32_t i) const {
        const uint32_t key = skeys[idx ? idx[i] : i];
        const uint32_t z = key / sxy, rem = key - z * sxy, y = rem / sx, x = rem - y * sx;
        return ((z >> 2) * ty + (y >> 2)) * tx + (x >> 2);
    }
};

template <class Tile>
__global__ void __launch_bounds__(256) k_tile_count(Tile tile, const uint32_t* __restrict__ n_dev, uint32_t n_host,
                                                    uint32_t* __restrict__ tile_count, uint32_t* __restrict__ tid_of,
                                                    uint32_t* __restrict__ slot) {
    const uint32_t n = n_dev ? *n_dev : n_host;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t t = tile(i);
        tid_of[i] = t;
        slot[i] = atomicAdd(&tile_count[t], 1u);
    }
}

__global__ void __launch_bounds__(256) k_tile_scatter(const uint32_t* __restrict__ n_dev, uint32_t n_host,
                                                      const uint32_t* __restrict__ tile_start,
                                                      const uint32_t* __restrict__ tid_of,
                                                      const uint32_t* __restrict__ slot, uint32_t* __restrict__ perm) {
    const uint32_t n = n_dev ? *n_dev : n_host;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        perm[tile_start[tid_of[i]] + slot[i]] = i;
}

template <class Tile>
static pms_status tile_perm(pms_ctx* ctx, Tile tile, uint64_t ntiles, const uint32_t* n_dev, uint32_t n_host,
                            pms::OrderBufs& ob) {
    pms_status st0 = ensure_order(ctx, ob, n_host, ntiles);   // a no-op once sized (batches size them first)
    if (st0) return st0;
    PMS_CUDA(ctx, cudaMemsetAsync(ob.tile_count.p, 0, 4 * ntiles, ctx->stream));
    k_tile_count<<<grid_for(n_host, 256), 256, 0, ctx->stream>>>(tile, n_dev, n_host, ob.tile_count.as<uint32_t>(),
                                                                 ob.tid_of.as<uint32_t>(), ob.slot.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    pms_status st = scan_u32(ctx, ob.tile_count.as<uint32_t>(), ob.tile_start.as<uint32_t>(), ntiles, nullptr);
    if (st) return st;
    k_tile_scatter<<<grid_for(n_host, 256), 256, 0, ctx->stream>>>(n_dev, n_host, ob.tile_start.as<uint32_t>(),
                                                                   ob.tid_of.as<uint32_t>(), ob.slot.as<uint32_t>(),
                                                                   ob.perm.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

uint64_t vertex_tiles(const pms_grid& g) {
    return (uint64_t)((g.scres[0] + 7) >> 3) * ((g.scres[1] + 7) >> 3) * ((g.scres[2] + 7) >> 3);
}
uint64_t particle_tiles(const pms_grid& g) {
    return (uint64_t)((g.spres[0] + 3) >> 2) * ((g.spres[1] + 3) >> 2) * ((g.spres[2] + 3) >> 2);
}

pms_status ensure_order(pms_ctx* ctx, pms::OrderBufs& ob, uint64_t items, uint64_t ntiles) {
    const size_t I = items ? items : 1, T = ntiles ? ntiles : 1;
    PMS_CUDA(ctx, ob.perm.ensure(4 * I));
    PMS_CUDA(ctx, ob.tid_of.ensure(4 * I));
    PMS_CUDA(ctx, ob.slot.ensure(4 * I));
    PMS_CUDA(ctx, ob.tile_count.ensure(4 * T));
    PMS_CUDA(ctx, ob.tile_start.ensure(4 * T));
    return PMS_OK;
}

// band vertices vlist[0 .. *n_dev) (n_host: a bound) in vertex-tile order
pms_status launch_vertex_order(pms_ctx* ctx, const uint32_t* vlist, const uint32_t* n_dev, uint32_t n_host) {
    const pms_grid& g = ctx->grid;
    VertexTile t{vlist, g.scres[0], g.scres[0] * g.scres[1], (g.scres[0] + 7) >> 3, (g.scres[1] + 7) >> 3};
    return tile_perm(ctx, t, vertex_tiles(g), n_dev, n_host, ctx->vorder);
}

// particles 0 .. n-1 in spatial-tile order
pms_status launch_particle_order(pms_ctx* ctx) {
    const pms_grid& g = ctx->grid;
    ParticleTile t{ctx->skeys.as<uint32_t>(), nullptr, g.spres[0], g.spres[0] * g.spres[1], (g.spres[0] + 3) >> 2,
                   (g.spres[1] + 3) >> 2};
    return tile_perm(ctx, t, particle_tiles(g), nullptr, ctx->n, ctx->porder);
}

// surface particles slist[0 .. ns) (bounded by n) in spatial-tile order
pms_status launch_surface_order(pms_ctx* ctx) {
    const pms_grid& g = ctx->grid;
    Counters* cnt = ctx->counters.as<Counters>();
    ParticleTile t{ctx->skeys.as<uint32_t>(), ctx->slist.as<uint32_t>(), g.spres[0], g.spres[0] * g.spres[1],
                   (g.spres[0] + 3) >> 2, (g.spres[1] + 3) >> 2};
    return tile_perm(ctx, t, particle_tiles(g), &cnt->ns, ctx->n, ctx->sorder);
}

}  // namespace pms
