/*
 * CPU restatement of the cornerstone-octree single-GPU path: SFC keys, stable key sort, cornerstone leaf build,
 * internal-tree link, node geometry, halo discovery and neighbour search.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the oracle that the CUDA path is checked against. The product
 * (the C-ABI library in cornerstone-octree_gb300/) never links, loads or calls it; only tests, the smoke check
 * and the CPU-baseline leg of the benchmark do.
 *
 * Keys of both widths are carried in uint64_t arrays; `key_bits` (32 or 64) selects the reference's 10- or
 * 21-level key arithmetic. Every function cites the reference function it restates.
 */
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* boundary: 0 open, 1 periodic, 2 fixed, 3 cubic_open (cstone::BoundaryType, sfc/box.hpp:77-83) */
typedef struct
{
    double lo[3];
    double hi[3];
    int boundary[3];
} cso_box;

enum { CSO_MORTON = 0, CSO_HILBERT = 1 };

/* ---- key algebra (sfc/common.hpp, sfc/morton.hpp, sfc/hilbert.hpp) ---- */
uint64_t cso_imorton(unsigned ix, unsigned iy, unsigned iz, int key_bits);
uint64_t cso_ihilbert(unsigned ix, unsigned iy, unsigned iz, int key_bits);
void cso_decode_morton(uint64_t key, int key_bits, unsigned* ixyz);
void cso_decode_hilbert(uint64_t key, int key_bits, unsigned* ixyz);

/* ---- keys (sfc/sfc.hpp:142-179, 268-283) ---- */
void cso_sfc_keys_f64(const double* x, const double* y, const double* z, uint64_t* keys, size_t n,
                      const cso_box* box, int kind, int key_bits, int respect_remove_key);
void cso_sfc_keys_f32(const float* x, const float* y, const float* z, uint64_t* keys, size_t n,
                      const cso_box* box, int kind, int key_bits, int respect_remove_key);

/* ---- stable sort by key (primitives/gather.hpp:42-74, std::stable_sort) ---- */
void cso_sort_by_key(uint64_t* keys, uint32_t* values, size_t n);
void cso_gather_f64(const uint32_t* perm, const double* in, double* out, size_t n);
void cso_gather_f32(const uint32_t* perm, const float* in, float* out, size_t n);

/* ---- cornerstone leaf array (tree/csarray.hpp) ---- */
void cso_find_search_bounds(int64_t first_idx, uint64_t target, const uint64_t* codes, int64_t n_codes,
                            int key_bits, int64_t* out_lo, int64_t* out_hi);
void cso_node_counts(const uint64_t* tree, uint32_t* counts, int32_t num_nodes, const uint64_t* keys, size_t n,
                     uint32_t max_count, int use_counts_as_guess, int key_bits);
int cso_rebalance_decision(const uint64_t* tree, const uint32_t* counts, int32_t num_nodes, unsigned bucket,
                           int32_t* ops, int key_bits);
int32_t cso_rebalance_tree(const uint64_t* tree, int32_t num_nodes, int32_t* ops, uint64_t* new_tree,
                           int32_t new_capacity, int key_bits);
/* one updateOctree step; tree/counts are in/out with capacity `capacity` leaves; returns converged flag,
 * or -1 if the new tree needs more than `capacity` leaves (then *num_nodes holds the required count) */
int cso_update_octree(const uint64_t* keys, size_t n, unsigned bucket, uint32_t max_count, uint64_t* tree,
                      uint32_t* counts, int32_t* num_nodes, int32_t capacity, int key_bits);
/* computeOctree from the root; returns number of leaves (or -needed if capacity too small) */
int32_t cso_compute_octree(const uint64_t* keys, size_t n, unsigned bucket, uint32_t max_count, uint64_t* tree,
                           uint32_t* counts, int32_t capacity, int key_bits, int* iterations);

/* ---- internal octree (tree/octree.hpp:55-196) ---- */
int32_t cso_binary_key_weight(uint64_t key, unsigned level, int key_bits);
void cso_build_octree(const uint64_t* leaves, int32_t num_leaves, int key_bits, uint64_t* prefixes,
                      int32_t* child_offsets, int32_t* parents, int32_t* level_range, int32_t* internal_to_leaf,
                      int32_t* leaf_to_internal);

/* ---- geometry (focus/source_center.hpp:145-158, sfc/box.hpp:318-335) ---- */
void cso_node_fp_centers_f64(const uint64_t* prefixes, int32_t num_nodes, int kind, int key_bits,
                             const cso_box* box, double* centers, double* sizes);
void cso_node_fp_centers_f32(const uint64_t* prefixes, int32_t num_nodes, int kind, int key_bits,
                             const cso_box* box, float* centers, float* sizes);

/* ---- halo discovery (focus/source_center.hpp:28-43, traversal/collisions.hpp:25-94) ---- */
void cso_search_boxes_f64(const double* x, const double* y, const double* z, const double* h,
                          const uint32_t* layout, int32_t first_leaf, int32_t last_leaf, double scale,
                          const int32_t* leaf_to_internal, const double* node_centers, double* search_centers,
                          double* search_sizes);
void cso_search_boxes_f32(const float* x, const float* y, const float* z, const float* h,
                          const uint32_t* layout, int32_t first_leaf, int32_t last_leaf, float scale,
                          const int32_t* leaf_to_internal, const float* node_centers, float* search_centers,
                          float* search_sizes);
void cso_find_halos_f64(const uint64_t* prefixes, const int32_t* child_offsets, const int32_t* parents,
                        const double* node_centers, const double* node_sizes, const uint64_t* leaves,
                        const double* search_centers, const double* search_sizes, const cso_box* box,
                        int32_t first_node, int32_t last_node, int key_bits, uint8_t* flags);
void cso_find_halos_f32(const uint64_t* prefixes, const int32_t* child_offsets, const int32_t* parents,
                        const float* node_centers, const float* node_sizes, const uint64_t* leaves,
                        const float* search_centers, const float* search_sizes, const cso_box* box,
                        int32_t first_node, int32_t last_node, int key_bits, uint8_t* flags);

/* ---- neighbour search (findneighbors.hpp:33-177) ---- */
void cso_find_neighbors_f64(const double* x, const double* y, const double* z, const double* h, uint32_t first,
                            uint32_t last, const cso_box* box, const int32_t* child_offsets,
                            const int32_t* parents, const int32_t* internal_to_leaf, const uint32_t* layout,
                            const double* centers, const double* sizes, float search_ext, unsigned ngmax,
                            uint32_t* neighbors, uint32_t* counts);
void cso_find_neighbors_f32(const float* x, const float* y, const float* z, const float* h, uint32_t first,
                            uint32_t last, const cso_box* box, const int32_t* child_offsets,
                            const int32_t* parents, const int32_t* internal_to_leaf, const uint32_t* layout,
                            const float* centers, const float* sizes, float search_ext, unsigned ngmax,
                            uint32_t* neighbors, uint32_t* counts);

void cso_find_neighbors_f64_hf32(const double* x, const double* y, const double* z, const float* h, uint32_t first,
                                 uint32_t last, const cso_box* box, const int32_t* child_offsets,
                                 const int32_t* parents, const int32_t* internal_to_leaf, const uint32_t* layout,
                                 const double* centers, const double* sizes, float search_ext, unsigned ngmax,
                                 uint32_t* neighbors, uint32_t* counts);
void cso_search_boxes_f64_hf32(const double* x, const double* y, const double* z, const float* h,
                               const uint32_t* layout, int32_t first_leaf, int32_t last_leaf, float scale,
                               const int32_t* leaf_to_internal, const double* node_centers, double* search_centers,
                               double* search_sizes);

/* ---- workload generators (seeded, counter-based; shared by every test and benchmark) ---- */
void cso_philox_uniform_f64(uint64_t seed, uint64_t stream, double* out, size_t n, double lo, double hi);
void cso_plummer_f64(uint64_t seed, double* x, double* y, double* z, size_t n, double rmax);
int cso_num_threads(void);

/* ---- around the path: upsweeps, source centres, groups, SFC gaps, focus rebalance (cs_oracle_next.inc) ---- */
int32_t cso_span_sfc_range(uint64_t a, uint64_t b, uint64_t* out, int key_bits);
int32_t cso_fill_sfc_gaps(const uint64_t* keys, int32_t num_nodes, uint64_t* out, int32_t cap, int key_bits);
void cso_upsweep_sum(const int32_t* level_range, int num_levels, const int32_t* child_offsets, uint32_t* counts);
void cso_leaf_mass_centers_f64(const double* x, const double* y, const double* z, const double* m,
                               const int32_t* leaf_to_internal, int32_t num_leaves, const uint32_t* layout,
                               double* centers);
void cso_leaf_mass_centers_f64m32(const double* x, const double* y, const double* z, const float* m,
                                  const int32_t* leaf_to_internal, int32_t num_leaves, const uint32_t* layout,
                                  double* centers);
void cso_leaf_mass_centers_f32(const float* x, const float* y, const float* z, const float* m,
                               const int32_t* leaf_to_internal, int32_t num_leaves, const uint32_t* layout,
                               float* centers);
void cso_upsweep_centers_f64(const int32_t* level_range, int num_levels, const int32_t* child_offsets,
                             double* centers);
void cso_upsweep_centers_f32(const int32_t* level_range, int num_levels, const int32_t* child_offsets,
                             float* centers);
int32_t cso_group_splits_f64(uint32_t first, uint32_t last, const double* x, const double* y, const double* z,
                             const double* h, const uint64_t* leaves, int32_t num_leaves, const uint32_t* layout,
                             const double* box_lo, const double* box_hi, unsigned group_size, float tol,
                             uint32_t* groups, int32_t cap, int key_bits);
int32_t cso_group_splits_f32(uint32_t first, uint32_t last, const float* x, const float* y, const float* z,
                             const float* h, const uint64_t* leaves, int32_t num_leaves, const uint32_t* layout,
                             const double* box_lo, const double* box_hi, unsigned group_size, float tol,
                             uint32_t* groups, int32_t cap, int key_bits);
void cso_rebalance_decision_essential(const uint64_t* prefixes, const int32_t* child_offsets, const int32_t* parents,
                                      const uint32_t* counts, const uint8_t* macs, int32_t num_nodes,
                                      uint64_t focus_start, uint64_t focus_end, unsigned bucket, int32_t* ops,
                                      int key_bits);
void cso_mac_refine_decision(const uint64_t* prefixes, const uint8_t* macs, const int32_t* l2i, int32_t num_leaves,
                             int32_t focus_first, int32_t focus_last, int32_t* ops, int key_bits);
int cso_protect_ancestors(const uint64_t* prefixes, const int32_t* parents, int32_t* ops, int32_t num_nodes,
                          int key_bits);
int cso_enforce_keys(const uint64_t* keys, int32_t n_keys, const uint64_t* prefixes, const int32_t* child_offsets,
                     const int32_t* parents, int32_t* ops, int key_bits);
void cso_range_count(const uint64_t* leaves, int32_t n_leaf_keys, const uint32_t* counts, const uint64_t* leaves_focus,
                     const int32_t* focus_idx, int32_t n_idx, uint32_t* counts_focus);
void cso_node_layout(const uint32_t* focus_leaf_counts, int32_t num_leaves, const uint8_t* flags, const int32_t* l2i,
                     int32_t first, int32_t last, uint32_t* layout);
void cso_ijloop_density_list_f64(const double* x, const double* y, const double* z, const double* h, const double* m,
                                 uint32_t first, uint32_t last, const cso_box* box, const uint32_t* nb,
                                 const uint32_t* nc, unsigned ngmax, double* rho);
void cso_ijloop_density_list_f32(const float* x, const float* y, const float* z, const float* h, const float* m,
                                 uint32_t first, uint32_t last, const cso_box* box, const uint32_t* nb,
                                 const uint32_t* nc, unsigned ngmax, float* rho);
void cso_ijloop_density_all_f64(const double* x, const double* y, const double* z, const double* h, const double* m,
                                uint32_t n, const cso_box* box, double* rho);
void cso_ijloop_density_all_f32(const float* x, const float* y, const float* z, const float* h, const float* m,
                                uint32_t n, const cso_box* box, float* rho);

#ifdef __cplusplus
}
#endif
