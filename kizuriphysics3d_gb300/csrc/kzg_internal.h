// kzg_internal.h - functions shared between the translation units of libkzg (not exported).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>
#include <vector_types.h>

#include "../../include/kzg.h"

namespace kzg {

struct Ctx;

size_t cub_temp_bytes(uint32_t max_items);
cudaError_t configure_kernels();  // per-device kernel attributes (large dynamic shared memory)
// Packed-item scratch of the cluster solve for `points` point rows: entries per cluster island
// (cap) and float4 elements to allocate.
size_t pack_elements(uint32_t points, uint32_t* cap);
size_t cluster_id_words(uint32_t max_cons);  // local-id scratch of the cluster solve
cudaError_t init_new_bodies(Ctx& ctx, uint32_t first, uint32_t n);  // fat bounds, activity, active list of new bodies
cudaError_t set_bodies_active(Ctx& ctx, const uint32_t* dev_ids, uint32_t n, int active);  // in order
cudaError_t edit_bodies(Ctx& ctx, const kzg_body_edit* dev_edits, uint32_t n);  // in order
cudaError_t create_joints(Ctx& ctx, uint32_t first, uint32_t n);     // joint records from ctx.joint_stage
size_t joint_record_bytes();
size_t gjk_record_bytes();  // one kept GJK result of a pair deferred to the EPA pass
// Manifold cache table: room for `entries` at below 0.7 load (doubling, entries rehashed), and a
// table of exactly `cap` slots with every entry cleared (snapshot loads).
kzg_status cache_reserve(Ctx& ctx, uint64_t entries);
// The last step's WorldStats::numIslands with sleeping on, counted as the reference does; call
// before reading the stats and before anything changes the active list, the bodies or the joints.
kzg_status settle_sleep_count(Ctx& ctx);
kzg_status cache_reset(Ctx& ctx, uint32_t cap);
// Entries (slot, key, point count, 4 positions, 4 impulses) written into their slots.
kzg_status cache_scatter(Ctx& ctx, const uint32_t* slots, const unsigned long long* keys, const uint32_t* np,
                         const float4* pos, const float4* imp, uint32_t n);
kzg_status upload_forces(Ctx& ctx, const float* host_ft, uint32_t first, uint32_t n);          // 6 floats per body
kzg_status download_transforms(Ctx& ctx, float* host_out, uint32_t first, uint32_t n);      // 7 floats per body
kzg_status step_canonical(Ctx& ctx, float dt, uint32_t nsteps);
kzg_status step_external(Ctx& ctx, const uint32_t* host_pairs, uint32_t num_pairs, float dt);
kzg_status hash_state(Ctx& ctx, uint64_t* out);

// learned warm start (kzg_mlp.cu)
cudaError_t mlp_configure_kernels();
void mlp_free(Ctx& ctx);
kzg_status mlp_set_params(Ctx& ctx, const float* theta, const float* mean, const float* stdv);
kzg_status mlp_get_params(Ctx& ctx, float* theta, float* mean, float* stdv);
kzg_status mlp_log_begin(Ctx& ctx, uint32_t capacity);
kzg_status mlp_log_fetch(Ctx& ctx, float* out, uint32_t cap, uint32_t* n);
kzg_status mlp_set_dataset(Ctx& ctx, const float* samples, uint32_t n);
kzg_status mlp_gradient(Ctx& ctx, uint32_t first, uint32_t count, float* grad, float* loss);
kzg_status mlp_train_step(Ctx& ctx, uint32_t first, uint32_t count, float lr, float* loss);
kzg_status mlp_predict(Ctx& ctx, uint32_t first, uint32_t count, float* out);
uint32_t mlp_after_prepare(Ctx& ctx, float dt);  // kernels launched
uint32_t mlp_after_solve(Ctx& ctx, float dt);

// host setup (kzg_hull.cpp)
int hull_build(const float* pts, uint32_t n, uint32_t max_points, float* out_v, uint32_t* out_nv, uint8_t* out_sizes,
               uint32_t* out_nf, uint32_t* out_idx, uint32_t* out_ni, uint32_t cap_faces);
void mass_properties(const kzg_shape_desc& s, const float* hull_vertices, const uint8_t* face_sizes,
                     const uint32_t* face_indices, uint32_t motion, float density, float mass_override,
                     float* out_inv_mass, float* out_iil);
void shape_local_bounds(const kzg_shape_desc& s, const float* hull_vertices, float* mn, float* mx);

}  // namespace kzg
