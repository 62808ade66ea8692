/*
 * pms_oracle.h -- CPU oracle for the particle-to-surface pipeline.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * (xiaoxiaoyu1872/PostMPS, "VisFluid") algorithm, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * The product (postmps_gb300, libpms) never links, loads or calls it.
 *
 * Precision contract:
 *   - integer stages (grid parameters, cell keys, stable sort, cell ranges,
 *     surface cells, surface-particle list, band bitmap given normals/flags,
 *     marching-cubes case indices given the field) are restated bit-exactly,
 *     with the same float32 operations as the reference where a float result
 *     feeds an integer decision;
 *   - floating-point stages (density, weighted mean, covariance, eigen
 *     decomposition, G matrices, scalar field, mesh vertices) are evaluated in
 *     float64 ("FP64 oracle").
 *
 * Every function cites the reference file:line it follows.  Arrays are flat,
 * caller-owned; "pos" arrays are xyz-interleaved float32.
 */
#ifndef PMS_ORACLE_H
#define PMS_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Raw config.txt values (before derivation), as INIReader returns them.
 * Params.cpp:31-106. */
typedef struct orc_config {
    double mass;                    /* [Sim] Mass                        */
    double particle_spacing;        /* [Sim] ParticleSpacing             */
    double smoothing_radius_ratio;  /* [Surface] SmoothingRadiusRatio    */
    long   min_num_neighbors;       /* [Surface] MinNumNeighbors         */
    long   isolate_num_neighbors;   /* [Surface] IsolateNumNeighbors     */
    double lambda_for_smoothed;     /* [Surface] LambdaForSmoothed       */
    double iso_value;               /* [Surface] IsoValue                */
    double min_wave_crests, max_wave_crests;
    double min_trapped_air, max_trapped_air;
    double min_kinetic_energy, max_kinetic_energy;
    double trapped_air_multiplier, wave_crests_multiplier;
    double time_step, life_time, buoyancy_control, drag_control;
    double sp_scale, sc_scale;      /* [Domain] Spatial/SclarGridSizeScale */
} orc_config;

/* Derived parameters, float32 like the reference's structs (Define.h:85-139). */
typedef struct orc_params {
    float mass, particle_spacing;
    int   smoothing_radius_ratio;
    float h, h_inv, h_sq, aniso_radius;
    int   min_num_neighbors, isolate_num_neighbors;
    float lambda_for_smoothed, iso_value;
    /* diffuse */
    float hd, hd_inv, hd_sq, hd_aniso, coefficient;
    int   d_min_num_neighbors;
    float min_wc, max_wc, min_ta, max_ta, min_ke, max_ke;
    int   ta_mult, wc_mult, life_time;
    float time_step, buoyancy, drag;
    /* grid constants */
    int   sp_scale, sc_scale;
    float sp_grid_size, sc_grid_size;
    int   spexpand, scexpand, spexpand_diffuse;
} orc_params;

/* Per-frame grid (GridParams, Define.h:142-174, filled by FileData.cpp:259-279). */
typedef struct orc_grid {
    float min_pos[3], max_pos[3];
    float scmin_pos[3], scmax_pos[3];
    float sp_grid_size, sc_grid_size;
    uint32_t spres[3], scres[3];
    int32_t spexpand, scexpand, spexpand_diffuse;
    uint32_t sp_size, sc_size;
} orc_grid;

/* ---- parameters and grid ------------------------------------------------ */
void orc_derive_params(const orc_config* cfg, orc_params* out);
void orc_bbox(const float* pos, uint32_t n, float bmin[3], float bmax[3]);
void orc_grid_from_bbox(const orc_params* p, const float bmin[3], const float bmax[3], orc_grid* g);

/* ---- spatial hashing ------------------------------------------------------ */
void orc_hash(const orc_grid* g, const float* pos, uint32_t n, uint32_t* keys);
void orc_stable_sort(const uint32_t* keys, uint32_t n, uint32_t nkeys, uint32_t* perm);
void orc_cell_ranges(const uint32_t* sorted_keys, uint32_t n, uint32_t nkeys,
                     uint32_t* start, uint32_t* end);

/* ---- surface particles ----------------------------------------------------- */
void orc_surface_cells(const orc_grid* g, const uint32_t* start, const uint32_t* end,
                       uint32_t* surf_count);
uint64_t orc_exclusive_scan_u32(const uint32_t* in, uint64_t n, uint32_t* out);
void orc_surface_list(const orc_grid* g, const uint32_t* surf_count, const uint32_t* surf_scan,
                      const uint32_t* start, uint32_t* list);

/* ---- anisotropy (float64) ---------------------------------------------------- */
/* estimationOfScalarValue at mesh vertices (float64); out 5 per vertex {vel xyz, |vel|, rhop} */
void orc_scalar_values(const orc_params* p, const orc_grid* g, const float* spos, const float* svel,
                       const double* rho, const uint32_t* start, const uint32_t* end, const float* verts,
                       uint64_t m, double* out);
void orc_density(const orc_params* p, const orc_grid* g, const float* spos, uint32_t n,
                 const uint32_t* start, const uint32_t* end, double* rho);
/* Per surface particle s (list[s] = sorted index):
 *   mean[3s..]   weighted mean
 *   G[9s..]      row-major anisotropy matrix, maxv[s] = sigma_max/scale
 *   nrm[3s..]    oriented normal, flag[s] thin-feature/isolated flag
 *   nnb[s]       neighbour count within h                                       */
void orc_anisotropy(const orc_params* p, const orc_grid* g, const float* spos, uint32_t n,
                    const uint32_t* start, const uint32_t* end,
                    const uint32_t* list, uint32_t ns,
                    double* mean, double* G, double* maxv, double* nrm, uint8_t* flag,
                    uint32_t* nnb);

/* ---- narrow band (bit-exact given float32 normals and flags) ---------------- */
/* bitmap: ceil(sc_size/32) words, zeroed by the caller.  nrm/flag are the
 * float32 normal and flag of each surface particle (list order).            */
void orc_band_bitmap(const orc_grid* g, float h, const float* spos, const uint32_t* list,
                     uint32_t ns, const float* nrm, const uint8_t* flag, uint32_t* bitmap);
uint64_t orc_bitmap_to_list(const uint32_t* bitmap, uint64_t nbits, uint32_t* list);

/* ---- scalar field (float64) ------------------------------------------------ */
/* Gs: surface-particle G (9/particle, float64), maxv: sigma_max/scale.  rho:
 * density per sorted particle.  Writes field[v] for each band vertex.       */
void orc_field(const orc_params* p, const orc_grid* g, const float* spos, uint32_t n,
               const double* rho, const uint32_t* start, const uint32_t* end,
               const uint32_t* surf_count, const uint32_t* surf_scan,
               const double* Gs, const double* maxv,
               const uint32_t* verts, uint32_t nv, double* field);

/* ---- marching cubes -------------------------------------------------------- */
/* Tables must be installed once (from the test harness) before MC calls. */
void orc_mc_set_tables(const uint32_t* edge_flags /*256*/, const int32_t* tri /*256*16*/,
                       const uint32_t* num_vertices /*256*/, const uint32_t* edge_vertices /*24*/);
/* field_of(v) for band vertex list index i is fieldv[i]; band membership by bitmap.
 * Outputs per band vertex: cube case and vertex count; returns total mesh vertices. */
uint64_t orc_mc_classify(const orc_grid* g, float iso, const uint32_t* bitmap,
                         const uint32_t* verts, uint32_t nv, const float* fieldv,
                         uint32_t* cases, uint32_t* nvert);
/* Emits the triangle soup (float64 positions and normals) from a float64 field. */
void orc_mc_emit(const orc_grid* g, float iso, const uint32_t* bitmap,
                 const uint32_t* verts, uint32_t nv, const double* fieldv,
                 const uint32_t* cases, const uint32_t* nvert, const uint64_t* offsets,
                 double* vpos, double* vnrm);

/* ---- diffuse particles (pms_diffuse_oracle.c) ------------------------------- */
float orc_spawn_uniform(uint64_t seed, uint32_t frame, uint64_t idx);
void orc_df_normals(const orc_params* p, const orc_grid* g, const float* spos, uint32_t n,
                    const uint32_t* start, const uint32_t* end, uint32_t nfree, double* nrm);
void orc_df_trapped(const orc_params* p, const orc_grid* g, const float* spos, const float* svel, uint32_t n,
                    const uint32_t* start, const uint32_t* end, double* ita, double* energy);
void orc_df_crests(const orc_params* p, const orc_grid* g, const float* spos, const float* svel,
                   const uint32_t* start, const uint32_t* end, const uint32_t* free_list, uint32_t nfree,
                   const float* nrm, double* wc);
void orc_df_counts(const orc_params* p, const float* pot_raw, uint32_t n, float* pot_clamped, int32_t* num);
void orc_df_counts_from_clamped(const orc_params* p, const float* pot_clamped, uint32_t n, int32_t* num);
uint64_t orc_df_spawn(const orc_params* p, const orc_grid* g, const float* spos, const float* svel, uint32_t n,
                      const uint32_t* start, const uint32_t* end, const int32_t* num, uint64_t seed, uint32_t frame,
                      float* gen);
void orc_df_update(const orc_params* p, const orc_grid* g, const float* spos, const float* svel,
                   const uint32_t* start, const uint32_t* end, float* rec, uint32_t n_old);

/* ---- mesh comparison ------------------------------------------------------- */
/* One-sided Hausdorff distance from the vertices of soup A to the triangles
 * of soup B (both xyz float64, 3 vertices per triangle).                     */
double orc_hausdorff_vertices_to_mesh(const double* a, uint64_t na, const double* b, uint64_t nb,
                                      double cell);

#ifdef __cplusplus
}
#endif
#endif
