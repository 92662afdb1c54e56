// kzg_api.cu - the exported C-ABI (include/kzg.h): context lifetime, scene upload, stepping entry
// points and state/diagnostic downloads.  Every call returns a kzg_status and leaves a message
// in kzg_last_error() on failure; no C++ exception crosses the boundary.
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "kzg_ctx.h"
#include "kzg_internal.h"

using namespace kzg;

namespace {

std::string g_create_error;

#define CK(x)                                                            \
    do {                                                                 \
        cudaError_t e_ = (x);                                            \
        if (e_ != cudaSuccess) {                                         \
            ctx->err = std::string(#x) + ": " + cudaGetErrorString(e_);  \
            return KZG_ERR_CUDA;                                         \
        }                                                                \
    } while (0)
// The last step's sleeping island count is counted before the stats are read or anything it reads
// changes (settle_sleep_count).
#define SETTLE(c)                                        \
    do {                                                 \
        const kzg_status st_ = settle_sleep_count(*(c)); \
        if (st_ != KZG_OK) return st_;                   \
    } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
    return cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
}

kzg_status alloc_all(Ctx* ctx) {
    const kzg_config& c = ctx->cfg;
    const size_t B = c.max_bodies, P = c.max_pairs, R = 4ull * c.max_pairs, H = c.max_cache_entries;
    DeviceBodies& b = ctx->b;
    float4** f4b[] = {&b.pos, &b.rot, &b.lv, &b.av, &b.plv, &b.pav, &b.force, &b.torque, &b.prm0, &b.prm1,
                      &b.aabb_mn, &b.aabb_mx, &b.fat_mn, &b.fat_mx};
    for (float4** p : f4b) CK(dalloc(p, B));
    CK(dalloc(&b.iiw, 3 * B));
    CK(dalloc(&b.iil, 3 * B));
    CK(dalloc(&b.inv_mass, B));
    uint32_t** u32b[] = {&b.shape, &b.motion, &b.flags, &b.layer, &b.mask, &b.world, &b.packed, &b.act, &b.isl_idx,
                         &b.apos, &ctx->alist, &ctx->node, &ctx->dyn2slot, &ctx->act_flag, &ctx->act_scan, &ctx->suf,
                         &ctx->smin, &ctx->smark, &ctx->root_mark, &ctx->ccd_rank_keys, &ctx->ccd_sorted,
                         &ctx->ccd_keys_sorted};
    for (uint32_t** p : u32b) CK(dalloc(p, B));
    CK(dalloc(&b.sleep_t, B));
    CK(cudaMemset(b.plv, 0, sizeof(float4) * B));
    CK(cudaMemset(b.pav, 0, sizeof(float4) * B));
    CK(cudaMemset(b.force, 0, sizeof(float4) * B));
    CK(cudaMemset(b.torque, 0, sizeof(float4) * B));
    CK(dalloc(&ctx->is_large, B));
    CK(dalloc(&ctx->large_list, B));
    CK(dalloc(&ctx->large_off, 65537));  // world ids are < 65536
    CK(dalloc(&ctx->cell_keys, B));
    CK(dalloc(&ctx->cell_keys_sorted, B));
    CK(dalloc(&ctx->cell_vals, B));
    CK(dalloc(&ctx->cell_vals_sorted, B));
    CK(dalloc(&ctx->pair_keys, P));
    CK(dalloc(&ctx->pair_keys_sorted, P));
    CK(dalloc(&ctx->pairs, P));
    CK(dalloc(&ctx->m_count, P));
    CK(dalloc(&ctx->m_data, 12 * P));
    CK(dalloc(&ctx->m_key, P));
    CK(dalloc(&ctx->epa_list, P));
    ctx->epa_gjk_cap = (uint32_t)std::min<size_t>(P, size_t(1) << 20);
    CK(cudaMalloc(&ctx->epa_gjk, gjk_record_bytes() * std::max<size_t>(ctx->epa_gjk_cap, 1)));
    CK(dalloc(&ctx->ccd_disp, B));
    CK(dalloc(&ctx->ccd_list, B));
    CK(dalloc(&ctx->ccd_state, B));
    CK(dalloc(&ctx->ccd_deps, 8 * B));
    CK(dalloc(&ctx->ccd_ndeps, B));
    if (c.max_joints) {
        CK(cudaMalloc((void**)&ctx->joints, joint_record_bytes() * c.max_joints));
        CK(dalloc(&ctx->joint_stage, c.max_joints));
        CK(dalloc(&ctx->jkeys, c.max_joints));
        CK(dalloc(&ctx->jkeys_sorted, c.max_joints));
        CK(dalloc(&ctx->jisl, c.max_joints));
        CK(dalloc(&ctx->jisl_cisl, c.max_joints));
        CK(dalloc(&ctx->jflag, P + 1));
    }
    CK(dalloc(&ctx->con_flag, P));
    CK(dalloc(&ctx->con_index, P));
    CK(dalloc(&ctx->con_pair, P));
    CK(dalloc(&ctx->con_a, P));
    CK(dalloc(&ctx->con_b, P));
    CK(dalloc(&ctx->con_np, P));
    CK(dalloc(&ctx->con_bits, P));
    CK(dalloc(&ctx->con_fr, P));
    CK(dalloc(&ctx->con_key, P));
    DeviceRows& r = ctx->r;
    float4** rows[] = {&r.pA, &r.pB, &r.n, &r.t1, &r.t2, &r.rA, &r.rB, &r.rAr, &r.rBr, &r.laA, &r.laB,
                       &r.mass, &r.imp, &r.bias};
    for (float4** p : rows) {
        CK(dalloc(p, R));
        CK(cudaMemset(*p, 0, sizeof(float4) * R));
    }
    CK(dalloc(&ctx->uf, B));
    CK(dalloc(&ctx->isl_key, P));
    CK(dalloc(&ctx->isl_key_sorted, P));
    CK(dalloc(&ctx->isl_con_in, P));
    CK(dalloc(&ctx->isl_con, P));
    CK(dalloc(&ctx->isl_head, P));
    CK(dalloc(&ctx->isl_start, P + 1));
    CK(dalloc(&ctx->isl_pts, P));
    CK(dalloc(&ctx->lvl_count, R + P + 1));
    CK(dalloc(&ctx->brec, 4 * (R + P + 1)));
    CK(dalloc(&ctx->pk, pack_elements((uint32_t)std::min<size_t>(R, 0xFFFFFFFFu), &ctx->pk_cap)));
    CK(dalloc(&ctx->cl_ids, cluster_id_words((uint32_t)P)));
    CK(dalloc(&ctx->last_g, 3 * 2 * P));
    CK(dalloc(&ctx->first_w, P));
    CK(dalloc(&ctx->first_b, P));
    CK(dalloc(&ctx->lvl_tmp, R));
    CK(dalloc(&ctx->ids_tmp, R));
    CK(dalloc(&ctx->wl_list, R));
    CK(dalloc(&ctx->vl_list, R));
    CK(dalloc(&ctx->bl_list, R));
    CK(dalloc(&ctx->wl_off, R + P + 1));
    CK(dalloc(&ctx->vl_off, R + P + 1));
    CK(dalloc(&ctx->bl_off, R + P + 1));
    CK(dalloc(&ctx->isl_meta, 4 * P));
    CK(dalloc(&ctx->body_stamp, B));
    CK(cudaMemset(ctx->body_stamp, 0, sizeof(uint32_t) * B));
    CK(dalloc(&ctx->body_loc, B));
    CK(dalloc(&ctx->isl_bodies, 2 * P));
    CK(dalloc(&ctx->con_la, P));
    CK(dalloc(&ctx->con_lb, P));
    CK(dalloc(&ctx->isl_small, P));
    CK(dalloc(&ctx->isl_large, P));
    CK(dalloc(&ctx->isl_order, P));
    CK(dalloc(&ctx->isl_bins, 64));
    CK(dalloc(&ctx->miss_rows, R));
    CK(dalloc(&ctx->miss_prior, R));
    CK(configure_kernels());
    CK(dalloc(&ctx->c_key, H));
    CK(cudaMemset(ctx->c_key, 0, sizeof(unsigned long long) * H));
    CK(dalloc(&ctx->c_np, H));
    CK(dalloc(&ctx->c_pos, 4 * H));
    CK(dalloc(&ctx->c_imp, 4 * H));
    CK(cudaMemset(ctx->c_np, 0, sizeof(uint32_t) * H));
    ctx->cache_cap = (uint32_t)H;
    CK(dalloc(&ctx->dcnt, 1));
    CK(cudaMemset(ctx->dcnt, 0, sizeof(Counters)));
    CK(cudaMallocHost((void**)&ctx->hcnt, sizeof(Counters)));
    std::memset(ctx->hcnt, 0, sizeof(Counters));
    ctx->cub_tmp_bytes = cub_temp_bytes(std::max<uint32_t>(c.max_pairs, c.max_bodies));
    CK(cudaMalloc(&ctx->cub_tmp, ctx->cub_tmp_bytes));
    CK(dalloc(&ctx->hash_words, 14 * B));
    for (cudaEvent_t& e : ctx->ev) CK(cudaEventCreate(&e));
    return KZG_OK;
}

void free_all(Ctx* ctx) {
    DeviceBodies& b = ctx->b;
    void* ptrs[] = {b.act, b.sleep_t, b.isl_idx, b.apos, ctx->alist, ctx->node, ctx->dyn2slot, ctx->act_flag,
                    ctx->act_scan, ctx->suf, ctx->smin, ctx->smark, ctx->root_mark, ctx->ccd_rank_keys,
                    ctx->ccd_sorted, ctx->ccd_keys_sorted,
                    b.pos, b.rot, b.lv, b.av, b.plv, b.pav, b.force, b.torque, b.prm0, b.prm1, b.aabb_mn, b.aabb_mx,
                    b.iiw, b.iil, b.inv_mass, b.shape, b.motion, b.flags, b.layer, b.mask, b.world, b.packed, b.fat_mn, b.fat_mx,
                    ctx->is_large, ctx->large_list, ctx->large_off, ctx->cell_keys, ctx->cell_keys_sorted,
                    ctx->cell_vals, ctx->cell_vals_sorted, ctx->pair_keys, ctx->pair_keys_sorted, ctx->pairs,
                    ctx->m_count, ctx->m_data, ctx->m_key, ctx->epa_list, ctx->epa_gjk, ctx->ccd_disp, ctx->ccd_list, ctx->ccd_state, ctx->ccd_deps, ctx->ccd_ndeps, ctx->joints, ctx->joint_stage, ctx->jkeys,
                    ctx->jkeys_sorted, ctx->jisl, ctx->jisl_cisl, ctx->jflag, ctx->con_flag, ctx->con_index, ctx->con_pair, ctx->con_a,
                    ctx->con_b, ctx->con_np, ctx->con_bits, ctx->con_fr, ctx->con_key, ctx->r.pA, ctx->r.pB, ctx->r.n,
                    ctx->r.t1, ctx->r.t2, ctx->r.rA, ctx->r.rB, ctx->r.rAr, ctx->r.rBr, ctx->r.laA, ctx->r.laB,
                    ctx->r.mass, ctx->r.imp, ctx->r.bias, ctx->uf, ctx->isl_key, ctx->isl_key_sorted,
                    ctx->isl_con_in, ctx->isl_con, ctx->isl_head, ctx->isl_start, ctx->isl_pts, ctx->lvl_count,
                    ctx->brec, ctx->pk, ctx->cl_ids, ctx->last_g, ctx->first_w, ctx->first_b, ctx->lvl_tmp, ctx->ids_tmp,
                    ctx->wl_list, ctx->vl_list, ctx->bl_list, ctx->wl_off, ctx->vl_off, ctx->bl_off, ctx->isl_meta,
                    ctx->c_key, ctx->c_np, ctx->c_pos, ctx->c_imp, ctx->dcnt, ctx->cub_tmp, ctx->hash_words,
                    ctx->body_stamp, ctx->body_loc, ctx->isl_bodies, ctx->con_la, ctx->con_lb, ctx->isl_small,
                    ctx->isl_large, ctx->isl_order, ctx->isl_bins, ctx->miss_rows, ctx->miss_prior,
                    ctx->shapes, ctx->hull_verts, ctx->face_sizes, ctx->face_idx};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (ctx->hcnt) cudaFreeHost(ctx->hcnt);
    for (cudaEvent_t e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    mlp_free(*ctx);
}

struct HostShape {
    kzg_shape_desc d;
    float radius;  // bounds every rotated world-AABB half size of the shape
};

struct HostSide {
    std::vector<HostShape> shapes;
    std::vector<uint32_t> shape, motion, world;
    bool dirty = true;
};

}  // namespace

// Host-side mirror kept next to each context.
struct kzg_ctx {
    Ctx c;
    HostSide h;
};

namespace {

// Large bodies (planes, and bodies far larger than the typical one) bypass the uniform grid and
// are tested against every body of their world; the grid cell fits every other body's AABB.
kzg_status finalize_bodies(kzg_ctx* k) {
    Ctx* ctx = &k->c;
    HostSide& h = k->h;
    if (!h.dirty) return KZG_OK;
    ctx->graph_dirty = true;
    const uint32_t n = ctx->nbodies;
    std::vector<float> rad;
    for (uint32_t i = 0; i < n; ++i) {
        const HostShape& s = h.shapes[h.shape[i]];
        if (s.d.type != KZG_SHAPE_PLANE) rad.push_back(s.radius);
    }
    float r90 = 0.0f;
    if (!rad.empty()) {
        std::vector<float> t = rad;
        size_t q = (t.size() * 9) / 10;
        std::nth_element(t.begin(), t.begin() + q, t.end());
        r90 = t[q];
    }
    std::vector<uint8_t> large(n, 0);
    float rmax_small = 0.0f;
    uint32_t nworlds = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const HostShape& s = h.shapes[h.shape[i]];
        bool lg = s.d.type == KZG_SHAPE_PLANE || (r90 > 0.0f && s.radius > 4.0f * r90);
        large[i] = lg ? 1 : 0;
        if (!lg) rmax_small = std::max(rmax_small, s.radius);
        nworlds = std::max(nworlds, h.world[i] + 1);
    }
    ctx->cell_size = rmax_small > 0.0f ? 2.02f * rmax_small : 1.0f;
    std::vector<uint32_t> off(nworlds + 1, 0), list;
    for (uint32_t i = 0; i < n; ++i)
        if (large[i]) off[h.world[i] + 1]++;
    for (uint32_t w = 0; w < nworlds; ++w) off[w + 1] += off[w];
    list.resize(off[nworlds]);
    std::vector<uint32_t> fill(off.begin(), off.end() - 1);
    for (uint32_t i = 0; i < n; ++i)
        if (large[i]) list[fill[h.world[i]]++] = i;
    ctx->nlarge = (uint32_t)list.size();
    ctx->nworlds = nworlds;
    CK(cudaMemcpy(ctx->is_large, large.data(), n, cudaMemcpyHostToDevice));
    if (!list.empty()) CK(cudaMemcpy(ctx->large_list, list.data(), sizeof(uint32_t) * list.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->large_off, off.data(), sizeof(uint32_t) * off.size(), cudaMemcpyHostToDevice));
    h.dirty = false;
    return KZG_OK;
}

kzg_status check(kzg_ctx* c) { return c ? KZG_OK : KZG_ERR_INVALID; }
}  // namespace

extern "C" {

void kzg_default_settings(kzg_world_settings* ws, kzg_solver_settings* ss) {
    if (ws) {
        ws->gravity[0] = 0.0f; ws->gravity[1] = -9.81f; ws->gravity[2] = 0.0f;
        ws->fixed_timestep = (float)(1.0 / 60.0);
        ws->allow_sleeping = 1;  // WorldSettings::allowSleeping (PhysicsWorld.h:24)
        ws->warm_start = 1;
        ws->use_ccd = 1;                 // WorldSettings defaults, PhysicsWorld.h:39-42
        ws->ccd_max_penetration = 0.01f;
        ws->sleep_time_threshold = 0.5f;  // PhysicsWorld.h:25-27
        ws->sleep_linear_threshold = 0.05f;
        ws->sleep_angular_threshold = 0.1f;
    }
    if (ss) {  // SolverSettings defaults, ContactSolver.h:67-82
        ss->velocity_iterations = 16;
        ss->position_iterations = 6;
        ss->baumgarte = 0.2f;
        ss->penetration_slop = 0.005f;
        ss->restitution_threshold = 1.0f;
        ss->max_bias_velocity = 3.0f;
        ss->warm_start_factor = 1.0f;
        ss->use_velocity_bias = 0;
        ss->schedule = KZG_SCHEDULE_REFERENCE;
        ss->residual_tolerance = 0.0f;
        ss->max_velocity_iterations = 64;
        ss->use_split_impulse = 1;
        ss->use_simd_solver = 1;
    }
}

kzg_status kzg_create(const kzg_config* cfg, kzg_ctx** out) {
    if (!cfg || !out) { g_create_error = "null argument"; return KZG_ERR_INVALID; }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        g_create_error = "no CUDA device: the contact pipeline has no CPU fallback";
        return KZG_ERR_CUDA;
    }
    if (cfg->device < 0 || cfg->device >= ndev) { g_create_error = "bad device ordinal"; return KZG_ERR_INVALID; }
    if (cfg->max_cache_entries == 0 || (cfg->max_cache_entries & (cfg->max_cache_entries - 1)) != 0) {
        g_create_error = "max_cache_entries must be a power of two";
        return KZG_ERR_INVALID;
    }
    if (cfg->max_bodies == 0 || cfg->max_bodies > 0x00FFFFFFu || cfg->max_pairs == 0) {
        g_create_error = "max_bodies must be in [1, 2^24) and max_pairs > 0";
        return KZG_ERR_INVALID;
    }
    kzg_ctx* k = new (std::nothrow) kzg_ctx();
    if (!k) { g_create_error = "out of host memory"; return KZG_ERR_INVALID; }
    Ctx* ctx = &k->c;
    ctx->cfg = *cfg;
    ctx->device = cfg->device;
    kzg_default_settings(&ctx->ws, &ctx->ss);
    if (cudaSetDevice(cfg->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        g_create_error = "cannot open the CUDA device";
        delete k;
        return KZG_ERR_CUDA;
    }
    ctx->own_stream = true;
    kzg_status s = alloc_all(ctx);
    if (s != KZG_OK) {
        g_create_error = ctx->err;
        free_all(ctx);
        delete k;
        return s;
    }
    *out = k;
    return KZG_OK;
}

kzg_status kzg_destroy(kzg_ctx* k) {
    if (!k) return KZG_ERR_INVALID;
    cudaSetDevice(k->c.device);
    cudaStreamSynchronize(k->c.stream);
    free_all(&k->c);
    delete k;
    return KZG_OK;
}

const char* kzg_last_error(const kzg_ctx* k) { return k ? k->c.err.c_str() : g_create_error.c_str(); }

kzg_status kzg_set_stream(kzg_ctx* k, void* stream) {
    if (k) k->c.graph_dirty = true;
    if (check(k)) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    ctx->own_stream = false;
    ctx->stream = (cudaStream_t)stream;
    if (!stream) {
        CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->own_stream = true;
    }
    return KZG_OK;
}

kzg_status kzg_synchronize(kzg_ctx* k) {
    if (check(k)) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    CK(cudaStreamSynchronize(ctx->stream));
    return KZG_OK;
}

kzg_status kzg_set_world_settings(kzg_ctx* k, const kzg_world_settings* s) {
    if (k) k->c.graph_dirty = true;
    if (check(k) || !s) return KZG_ERR_INVALID;
    if (!(s->sleep_time_threshold >= 0.0f) || !(s->sleep_linear_threshold >= 0.0f) ||
        !(s->sleep_angular_threshold >= 0.0f)) {
        k->c.err = "sleep thresholds must be >= 0";
        return KZG_ERR_INVALID;
    }
    k->c.ws = *s;
    return KZG_OK;
}

kzg_status kzg_set_solver_settings(kzg_ctx* k, const kzg_solver_settings* s) {
    if (k) k->c.graph_dirty = true;
    if (check(k) || !s) return KZG_ERR_INVALID;
    if (s->schedule != KZG_SCHEDULE_REFERENCE) {
        k->c.err = "unknown solver schedule";
        return KZG_ERR_INVALID;
    }
    if (!(s->residual_tolerance >= 0.0f) || (s->residual_tolerance > 0.0f && s->max_velocity_iterations == 0)) {
        k->c.err = "residual_tolerance must be >= 0, with max_velocity_iterations >= 1 when it is > 0";
        return KZG_ERR_INVALID;
    }
    k->c.ss = *s;
    return KZG_OK;
}

kzg_status kzg_upload_shapes(kzg_ctx* k, const kzg_shape_desc* shapes, uint32_t ns, const float* hv, uint32_t nv,
                             const uint8_t* fs, uint32_t nf, const uint32_t* fi, uint32_t ni) {
    if (check(k) || (ns && !shapes)) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    if (ctx->shapes_uploaded) { ctx->err = "shapes are uploaded once per context"; return KZG_ERR_INVALID; }
    if (ns > ctx->cfg.max_shapes || nv > ctx->cfg.max_hull_vertices || ni > ctx->cfg.max_hull_indices) {
        ctx->err = "shape tables exceed kzg_config capacities";
        return KZG_ERR_CAPACITY;
    }
    std::vector<ShapeDev> dev(ns);
    HostSide& h = k->h;
    h.shapes.resize(ns);
    for (uint32_t i = 0; i < ns; ++i) {
        const kzg_shape_desc& d = shapes[i];
        if (d.type != KZG_SHAPE_SPHERE && d.type != KZG_SHAPE_BOX && d.type != KZG_SHAPE_CAPSULE &&
            d.type != KZG_SHAPE_HULL && d.type != KZG_SHAPE_PLANE) {
            ctx->err = "shape " + std::to_string(i) + ": type outside the accelerated set";
            return KZG_ERR_UNSUPPORTED;
        }
        if (d.type == KZG_SHAPE_HULL) {
            bool ok = d.num_vertices > 0 && d.num_faces > 0 && d.first_vertex + d.num_vertices <= nv &&
                      d.first_face + d.num_faces <= nf && d.first_index + d.num_indices <= ni && hv && fs && fi;
            uint64_t total = 0;
            for (uint32_t f = 0; ok && f < d.num_faces; ++f) {
                ok = fs[d.first_face + f] >= 3;
                total += fs[d.first_face + f];
            }
            ok = ok && total == d.num_indices;
            for (uint32_t q = 0; ok && q < d.num_indices; ++q) ok = fi[d.first_index + q] < d.num_vertices;
            if (!ok) {
                ctx->err = "shape " + std::to_string(i) + ": inconsistent hull ranges, face sizes or indices";
                return KZG_ERR_INVALID;
            }
        }
        ShapeDev& s = dev[i];
        std::memset(&s, 0, sizeof s);
        s.type = d.type;
        s.vfirst = d.first_vertex; s.vnum = d.num_vertices;
        s.ffirst = d.first_face; s.fnum = d.num_faces;
        s.ifirst = d.first_index; s.inum = d.num_indices;
        for (int q = 0; q < 4; ++q) s.p[q] = d.params[q];
        shape_local_bounds(d, hv, s.lmn, s.lmx);
        h.shapes[i].d = d;
        float ex = 0.5f * (s.lmx[0] - s.lmn[0]), ey = 0.5f * (s.lmx[1] - s.lmn[1]), ez = 0.5f * (s.lmx[2] - s.lmn[2]);
        float cx = 0.5f * (s.lmx[0] + s.lmn[0]), cy = 0.5f * (s.lmx[1] + s.lmn[1]), cz = 0.5f * (s.lmx[2] + s.lmn[2]);
        h.shapes[i].radius = std::sqrt(ex * ex + ey * ey + ez * ez) + std::sqrt(cx * cx + cy * cy + cz * cz);
    }
    CK(dalloc(&ctx->shapes, ns));
    CK(cudaMemcpy(ctx->shapes, dev.data(), sizeof(ShapeDev) * ns, cudaMemcpyHostToDevice));
    std::vector<float4> v4(nv);
    for (uint32_t i = 0; i < nv; ++i) v4[i] = make_float4(hv[3 * i], hv[3 * i + 1], hv[3 * i + 2], 0.0f);
    CK(dalloc(&ctx->hull_verts, nv));
    CK(dalloc(&ctx->face_sizes, nf));
    CK(dalloc(&ctx->face_idx, ni));
    if (nv) CK(cudaMemcpy(ctx->hull_verts, v4.data(), sizeof(float4) * nv, cudaMemcpyHostToDevice));
    if (nf) CK(cudaMemcpy(ctx->face_sizes, fs, nf, cudaMemcpyHostToDevice));
    if (ni) CK(cudaMemcpy(ctx->face_idx, fi, sizeof(uint32_t) * ni, cudaMemcpyHostToDevice));
    ctx->nshapes = ns;
    ctx->shapes_uploaded = true;
    return KZG_OK;
}

kzg_status kzg_add_bodies(kzg_ctx* k, uint32_t n, const kzg_body_soa* b, uint32_t* first_slot) {
    if (check(k) || !b) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    SETTLE(ctx);
    if (!ctx->shapes_uploaded) { ctx->err = "upload shapes before bodies"; return KZG_ERR_INVALID; }
    const uint32_t base = ctx->nbodies;
    if (base + n > ctx->cfg.max_bodies) { ctx->err = "kzg_config.max_bodies exceeded"; return KZG_ERR_CAPACITY; }
    if (!b->shape || !b->motion || !b->position || !b->rotation || !b->inv_mass || !b->inv_inertia_local) {
        ctx->err = "missing required body arrays";
        return KZG_ERR_INVALID;
    }
    HostSide& h = k->h;
    std::vector<float4> pos(n), rot(n), lv(n), av(n), p0(n), p1(n), iil(3 * n), iiw(3 * n);
    std::vector<uint32_t> flags(n), layer(n), mask(n), world(n), packed(n), motion(n), shape(n);
    for (uint32_t i = 0; i < n; ++i) {
        if (b->shape[i] >= ctx->nshapes || b->motion[i] > KZG_MOTION_DYNAMIC) {
            ctx->err = "body " + std::to_string(i) + ": bad shape index or motion type";
            return KZG_ERR_INVALID;
        }
        if (b->flags && (b->flags[i] & ~(KZG_BODY_SENSOR | KZG_BODY_ALLOW_SLEEPING | KZG_BODY_LINEAR_CAST))) {
            ctx->err = "unknown body flag";
            return KZG_ERR_INVALID;
        }
        auto f = [&](const float* a, uint32_t k_, float dflt) { return a ? a[k_] : dflt; };
        shape[i] = b->shape[i];
        motion[i] = b->motion[i];
        pos[i] = make_float4(b->position[3 * i], b->position[3 * i + 1], b->position[3 * i + 2], 0.0f);
        Quat q(b->rotation[4 * i], b->rotation[4 * i + 1], b->rotation[4 * i + 2], b->rotation[4 * i + 3]);
        rot[i] = make_float4(q.x, q.y, q.z, q.w);
        lv[i] = make_float4(f(b->linear_velocity, 3 * i, 0.0f), f(b->linear_velocity, 3 * i + 1, 0.0f),
                            f(b->linear_velocity, 3 * i + 2, 0.0f), 0.0f);
        av[i] = make_float4(f(b->angular_velocity, 3 * i, 0.0f), f(b->angular_velocity, 3 * i + 1, 0.0f),
                            f(b->angular_velocity, 3 * i + 2, 0.0f), 0.0f);
        // BodySettings defaults, Body.h:62-90
        p0[i] = make_float4(f(b->linear_damping, i, 0.05f), f(b->angular_damping, i, 0.05f),
                            f(b->gravity_factor, i, 1.0f), f(b->max_linear_velocity, i, 500.0f));
        p1[i] = make_float4(f(b->max_angular_velocity, i, 50.0f), f(b->friction, i, 0.5f), f(b->restitution, i, 0.0f),
                            f(b->ccd_motion_threshold, i, 0.0f));
        const float* L = b->inv_inertia_local + 9 * i;
        Mat3 IL{Vec3(L[0], L[1], L[2]), Vec3(L[3], L[4], L[5]), Vec3(L[6], L[7], L[8])};
        for (int c = 0; c < 3; ++c) iil[3 * i + c] = make_float4(L[3 * c], L[3 * c + 1], L[3 * c + 2], 0.0f);
        // World inertia at creation: MotionProperties::UpdateWorldInertia (Body.h:122-125) for
        // dynamic bodies with mass, zero otherwise (BodyManager.cpp:65-79).
        Mat3 W{Vec3(), Vec3(), Vec3()};
        if (motion[i] == KZG_MOTION_DYNAMIC && b->inv_mass[i] > 0.0f) {
            Mat3 R = q.to_mat3();
            W = (R * IL) * R.transposed();
        }
        iiw[3 * i] = make_float4(W.c0.x, W.c0.y, W.c0.z, 0.0f);
        iiw[3 * i + 1] = make_float4(W.c1.x, W.c1.y, W.c1.z, 0.0f);
        iiw[3 * i + 2] = make_float4(W.c2.x, W.c2.y, W.c2.z, 0.0f);
        flags[i] = b->flags ? b->flags[i] : KZG_BODY_ALLOW_SLEEPING;
        layer[i] = b->object_layer ? b->object_layer[i] : 1u;
        mask[i] = b->collision_mask ? b->collision_mask[i] : 0xFFFFFFFFu;
        world[i] = b->world_id ? b->world_id[i] : 0u;
        if (world[i] > 0xFFFFu) { ctx->err = "world_id must be < 65536"; return KZG_ERR_INVALID; }
        packed[i] = base + i;  // BodyID(index, sequence 0).Packed()
    }
    DeviceBodies& d = ctx->b;
    auto up4 = [&](float4* dst, const std::vector<float4>& src, size_t per) {
        return cudaMemcpy(dst + per * base, src.data(), sizeof(float4) * src.size(), cudaMemcpyHostToDevice);
    };
    auto up32 = [&](uint32_t* dst, const std::vector<uint32_t>& src) {
        return cudaMemcpy(dst + base, src.data(), sizeof(uint32_t) * src.size(), cudaMemcpyHostToDevice);
    };
    CK(up4(d.pos, pos, 1)); CK(up4(d.rot, rot, 1)); CK(up4(d.lv, lv, 1)); CK(up4(d.av, av, 1));
    CK(up4(d.prm0, p0, 1)); CK(up4(d.prm1, p1, 1)); CK(up4(d.iil, iil, 3)); CK(up4(d.iiw, iiw, 3));
    CK(cudaMemcpy(d.inv_mass + base, b->inv_mass, sizeof(float) * n, cudaMemcpyHostToDevice));
    CK(up32(d.shape, shape)); CK(up32(d.motion, motion)); CK(up32(d.flags, flags)); CK(up32(d.layer, layer));
    CK(up32(d.mask, mask)); CK(up32(d.world, world)); CK(up32(d.packed, packed));
    h.shape.insert(h.shape.end(), shape.begin(), shape.end());
    h.motion.insert(h.motion.end(), motion.begin(), motion.end());
    h.world.insert(h.world.end(), world.begin(), world.end());
    std::vector<uint32_t> cast;
    for (uint32_t i = 0; i < n; ++i)
        if (flags[i] & KZG_BODY_LINEAR_CAST) cast.push_back(base + i);
    if (!cast.empty()) {
        CK(cudaMemcpy(ctx->ccd_list + ctx->nccd, cast.data(), sizeof(uint32_t) * cast.size(), cudaMemcpyHostToDevice));
        ctx->nccd += (uint32_t)cast.size();
    }
    CK(init_new_bodies(*ctx, base, n));
    h.dirty = true;
    ctx->nbodies += n;
    if (first_slot) *first_slot = base;
    return KZG_OK;
}

kzg_status kzg_add_joints(kzg_ctx* k, uint32_t n, const kzg_joint_desc* j, uint32_t* first_index) {
    if (check(k) || (!j && n)) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    SETTLE(ctx);
    if (ctx->njoints + n > ctx->cfg.max_joints) { ctx->err = "kzg_config.max_joints exceeded"; return KZG_ERR_CAPACITY; }
    if (ctx->njoints + n > ctx->cfg.max_pairs) { ctx->err = "more joints than kzg_config.max_pairs"; return KZG_ERR_CAPACITY; }
    for (uint32_t i = 0; i < n; ++i) {
        if (j[i].type > KZG_JOINT_SIXDOF || j[i].body_a >= ctx->nbodies || j[i].body_b >= ctx->nbodies ||
            (j[i].flags & ~(KZG_JOINT_DISABLED | KZG_JOINT_LIMITS | KZG_JOINT_MOTOR | KZG_JOINT_LOCAL_ANCHORS))) {
            ctx->err = "joint " + std::to_string(i) + ": bad type, body slot or flag";
            return KZG_ERR_INVALID;
        }
    }
    if (n) {
        CK(cudaMemcpy(ctx->joint_stage, j, sizeof(kzg_joint_desc) * n, cudaMemcpyHostToDevice));
        CK(create_joints(*ctx, ctx->njoints, n));
    }
    if (first_index) *first_index = ctx->njoints;
    ctx->njoints += n;
    ctx->graph_dirty = true;
    return KZG_OK;
}

kzg_status kzg_step(kzg_ctx* k, float dt, uint32_t nsteps) {
    if (check(k)) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    if (!(dt > 0.0f)) return KZG_OK;  // PhysicsWorld::Step ignores dt <= 0 (PhysicsWorld.cpp:226)
    CK(cudaSetDevice(ctx->device));
    kzg_status s = finalize_bodies(k);
    if (s != KZG_OK) return s;
    if (nsteps == 0) return KZG_OK;
    return step_canonical(*ctx, dt, nsteps);
}

kzg_status kzg_set_tuning(kzg_ctx* k, const kzg_tuning* t) {
    if (check(k) || !t) return KZG_ERR_INVALID;
    if (t->small_island_constraints == 0 || t->small_island_constraints > 128 || t->warp_island_bodies == 0 ||
        t->warp_island_bodies > 384 || t->island_order > KZG_ISLANDS_LARGEST_FIRST) {
        k->c.err = "kzg_tuning: small_island_constraints in [1, 128], warp_island_bodies in [1, 384], "
                   "island_order KZG_ISLANDS_*";
        return KZG_ERR_INVALID;
    }
    k->c.tune = *t;
    k->c.graph_dirty = true;
    return KZG_OK;
}

kzg_status kzg_set_wait_limit(kzg_ctx* k, uint32_t polls) {
    if (check(k)) return KZG_ERR_INVALID;
    k->c.wait_limit = polls ? polls : kDefaultWaitLimit;
    k->c.graph_dirty = true;
    return KZG_OK;
}

kzg_status kzg_get_tuning(kzg_ctx* k, kzg_tuning* t) {
    if (check(k) || !t) return KZG_ERR_INVALID;
    *t = k->c.tune;
    return KZG_OK;
}

namespace {
// Device copy of everything a step changes that outlives the step (body state, world inertia, fat
// bounds, the manifold cache and its entry count, the joints), so that the tuner can time every
// candidate from one state and leave the world as it found it.
struct DeviceBackup {
    std::vector<std::pair<void*, size_t>> regions;
    uint8_t* mem = nullptr;

    cudaError_t save(Ctx& c) {
        const size_t nb = c.nbodies, H = c.cache_cap;
        DeviceBodies& b = c.b;
        for (float4* p : {b.pos, b.rot, b.lv, b.av, b.plv, b.pav, b.force, b.torque, b.fat_mn, b.fat_mx})
            regions.push_back({p, sizeof(float4) * nb});
        regions.push_back({b.iiw, sizeof(float4) * 3 * nb});
        regions.push_back({c.c_key, sizeof(unsigned long long) * H});
        regions.push_back({c.c_np, sizeof(uint32_t) * H});
        regions.push_back({c.c_pos, sizeof(float4) * 4 * H});
        regions.push_back({c.c_imp, sizeof(float4) * 4 * H});
        regions.push_back({&c.dcnt->cache_entries, sizeof(uint32_t)});
        regions.push_back({&c.dcnt->nact, sizeof(uint32_t)});
        for (void* p : {(void*)b.act, (void*)b.sleep_t, (void*)b.isl_idx, (void*)b.apos, (void*)c.alist})
            regions.push_back({p, sizeof(uint32_t) * nb});
        if (c.njoints) regions.push_back({c.joints, joint_record_bytes() * c.njoints});
        size_t total = 0;
        for (auto& r : regions) total += (r.second + 255) & ~size_t(255);
        cudaError_t e = cudaMalloc((void**)&mem, total ? total : 1);
        if (e != cudaSuccess) return e;
        return copy(c, true);
    }
    cudaError_t copy(Ctx& c, bool to_backup) {
        size_t off = 0;
        for (auto& r : regions) {
            void* dst = to_backup ? (void*)(mem + off) : r.first;
            const void* src = to_backup ? r.first : (const void*)(mem + off);
            cudaError_t e = cudaMemcpyAsync(dst, src, r.second, cudaMemcpyDeviceToDevice, c.stream);
            if (e != cudaSuccess) return e;
            off += (r.second + 255) & ~size_t(255);
        }
        return cudaStreamSynchronize(c.stream);
    }
    ~DeviceBackup() {
        if (mem) cudaFree(mem);
    }
};
}  // namespace

kzg_status kzg_autotune(kzg_ctx* k, float dt, uint32_t steps_per_candidate, kzg_tuning* best) {
    if (check(k) || !(dt > 0.0f) || steps_per_candidate == 0) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    CK(cudaSetDevice(ctx->device));
    SETTLE(ctx);
    kzg_status s = finalize_bodies(k);
    if (s != KZG_OK) return s;
    const kzg_tuning before = ctx->tune;
    // Every candidate starts from the saved state, so the cache never holds more than the entries
    // of 1 + steps_per_candidate steps beyond today's: reserve that, and keep the table (whose copy
    // the backup holds) in place while tuning.
    uint32_t entries = 0, pairs = 0;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&entries, &ctx->dcnt->cache_entries, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&pairs, &ctx->dcnt->npairs, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    s = cache_reserve(*ctx, (uint64_t)entries + (uint64_t)(steps_per_candidate + 1u) *
                                                    std::max<uint64_t>(std::max(pairs, ctx->nbodies), 1u));
    if (s != KZG_OK) return s;
    const bool logging = ctx->mlp.logging;
    ctx->mlp.logging = false;  // the tuning steps are not part of the world's history
    DeviceBackup backup;
    CK(backup.save(*ctx));
    const bool all_active = ctx->all_active;
    struct FixCache {
        Ctx* c;
        ~FixCache() { c->cache_fixed = false; }
    } fix{ctx};
    ctx->cache_fixed = true;
    const uint32_t small[3] = {32u, 64u, 128u}, warp[3] = {128u, 256u, 384u};
    const uint32_t orders[2] = {KZG_ISLANDS_IN_ORDER, KZG_ISLANDS_LARGEST_FIRST};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    kzg_tuning win{before.small_island_constraints, before.warp_island_bodies, 1e30f, before.island_order};
    for (uint32_t o = 0; o < 2 && s == KZG_OK; ++o)
        for (uint32_t a = 0; a < 3 && s == KZG_OK; ++a)
            for (uint32_t b = 0; b < 3 && s == KZG_OK; ++b) {
                kzg_tuning t{small[a], warp[b], 0.0f, orders[o]};
                ctx->tune = t;
                ctx->graph_dirty = true;
                ctx->all_active = all_active;
                if (backup.copy(*ctx, false) != cudaSuccess) { s = KZG_ERR_CUDA; break; }
                s = step_canonical(*ctx, dt, 1);  // first step of a choice: graph capture, not timed
                if (s != KZG_OK) break;
                cudaEventRecord(e0, ctx->stream);
                s = step_canonical(*ctx, dt, steps_per_candidate);
                cudaEventRecord(e1, ctx->stream);
                cudaEventSynchronize(e1);
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                t.step_ms = ms / (float)steps_per_candidate;
                if (t.step_ms < win.step_ms) win = t;
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const cudaError_t restored = backup.copy(*ctx, false);
    ctx->all_active = all_active;
    ctx->mlp.logging = logging;
    ctx->graph_dirty = true;
    if (s != KZG_OK) {
        ctx->tune = before;
        return s;
    }
    CK(restored);
    ctx->tune = win;
    if (best) *best = win;
    return KZG_OK;
}

kzg_status kzg_set_graph(kzg_ctx* k, int enabled) {
    if (check(k)) return KZG_ERR_INVALID;
    k->c.use_graph = enabled != 0;
    k->c.graph_dirty = true;
    return KZG_OK;
}

kzg_status kzg_step_with_pairs(kzg_ctx* k, const uint32_t* pairs, uint32_t np, float dt) {
    if (check(k) || (np && !pairs)) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    CK(cudaSetDevice(ctx->device));
    kzg_status s = finalize_bodies(k);
    if (s != KZG_OK) return s;
    return step_external(*ctx, pairs, np, dt);
}

kzg_status kzg_download_state(kzg_ctx* k, float* out, uint32_t first, uint32_t count) {
    if (check(k) || !out) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    if (first + count > ctx->nbodies) { ctx->err = "range outside the body array"; return KZG_ERR_INVALID; }
    std::vector<float4> p(count), q(count), l(count), a(count);
    CK(cudaMemcpyAsync(p.data(), ctx->b.pos + first, sizeof(float4) * count, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(q.data(), ctx->b.rot + first, sizeof(float4) * count, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(l.data(), ctx->b.lv + first, sizeof(float4) * count, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(a.data(), ctx->b.av + first, sizeof(float4) * count, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (uint32_t i = 0; i < count; ++i) {
        float* o = out + 13 * i;
        o[0] = p[i].x; o[1] = p[i].y; o[2] = p[i].z;
        o[3] = q[i].x; o[4] = q[i].y; o[5] = q[i].z; o[6] = q[i].w;
        o[7] = l[i].x; o[8] = l[i].y; o[9] = l[i].z;
        o[10] = a[i].x; o[11] = a[i].y; o[12] = a[i].z;
    }
    return KZG_OK;
}

kzg_status kzg_upload_state(kzg_ctx* k, const float* in, uint32_t first, uint32_t count) {
    if (check(k) || !in) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    if (first + count > ctx->nbodies) { ctx->err = "range outside the body array"; return KZG_ERR_INVALID; }
    std::vector<float4> p(count), q(count), l(count), a(count), il(3 * count), iw(3 * count);
    std::vector<float> im(count);
    CK(cudaMemcpy(il.data(), ctx->b.iil + 3ull * first, sizeof(float4) * 3 * count, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(im.data(), ctx->b.inv_mass + first, sizeof(float) * count, cudaMemcpyDeviceToHost));
    HostSide& h = k->h;
    for (uint32_t i = 0; i < count; ++i) {
        const float* s = in + 13 * i;
        p[i] = make_float4(s[0], s[1], s[2], 0.0f);
        q[i] = make_float4(s[3], s[4], s[5], s[6]);
        l[i] = make_float4(s[7], s[8], s[9], 0.0f);
        a[i] = make_float4(s[10], s[11], s[12], 0.0f);
        Mat3 W{Vec3(), Vec3(), Vec3()};
        if (h.motion[first + i] == KZG_MOTION_DYNAMIC && im[i] > 0.0f) {
            Quat qq(s[3], s[4], s[5], s[6]);
            Mat3 R = qq.to_mat3();
            Mat3 IL{Vec3(il[3 * i].x, il[3 * i].y, il[3 * i].z), Vec3(il[3 * i + 1].x, il[3 * i + 1].y, il[3 * i + 1].z),
                    Vec3(il[3 * i + 2].x, il[3 * i + 2].y, il[3 * i + 2].z)};
            W = (R * IL) * R.transposed();
        }
        iw[3 * i] = make_float4(W.c0.x, W.c0.y, W.c0.z, 0.0f);
        iw[3 * i + 1] = make_float4(W.c1.x, W.c1.y, W.c1.z, 0.0f);
        iw[3 * i + 2] = make_float4(W.c2.x, W.c2.y, W.c2.z, 0.0f);
    }
    CK(cudaMemcpy(ctx->b.pos + first, p.data(), sizeof(float4) * count, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->b.rot + first, q.data(), sizeof(float4) * count, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->b.lv + first, l.data(), sizeof(float4) * count, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->b.av + first, a.data(), sizeof(float4) * count, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->b.iiw + 3ull * first, iw.data(), sizeof(float4) * 3 * count, cudaMemcpyHostToDevice));
    return KZG_OK;
}

kzg_status kzg_download_transforms(kzg_ctx* k, float* out, uint32_t first, uint32_t count) {
    if (check(k) || !out) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    if (first + count > ctx->nbodies) { ctx->err = "range outside the body array"; return KZG_ERR_INVALID; }
    CK(cudaSetDevice(ctx->device));
    return download_transforms(*ctx, out, first, count);  // pos.xyz + rot.xyzw, 7 floats per body
}

kzg_status kzg_upload_forces(kzg_ctx* k, const float* ft, uint32_t first, uint32_t count) {
    if (check(k) || !ft) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    if (first + count > ctx->nbodies) { ctx->err = "range outside the body array"; return KZG_ERR_INVALID; }
    CK(cudaSetDevice(ctx->device));
    return upload_forces(*ctx, ft, first, count);
}

kzg_status kzg_download_mass(kzg_ctx* k, float* im, float* iw) {
    if (check(k)) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    const uint32_t n = ctx->nbodies;
    if (im) CK(cudaMemcpy(im, ctx->b.inv_mass, sizeof(float) * n, cudaMemcpyDeviceToHost));
    if (iw) {
        std::vector<float4> w(3ull * n);
        CK(cudaMemcpy(w.data(), ctx->b.iiw, sizeof(float4) * w.size(), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < w.size(); ++i) { iw[3 * i] = w[i].x; iw[3 * i + 1] = w[i].y; iw[3 * i + 2] = w[i].z; }
    }
    return KZG_OK;
}

kzg_status kzg_set_bodies_active(kzg_ctx* k, const uint32_t* packed_ids, uint32_t n, int active) {
    if (check(k) || (n && !packed_ids)) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    if (n == 0) return KZG_OK;
    CK(cudaSetDevice(ctx->device));
    SETTLE(ctx);
    if (n > ctx->cfg.max_pairs) { ctx->err = "more ids than kzg_config.max_pairs per call"; return KZG_ERR_CAPACITY; }
    CK(cudaMemcpyAsync(ctx->pair_keys, packed_ids, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(set_bodies_active(*ctx, reinterpret_cast<const uint32_t*>(ctx->pair_keys), n, active));
    if (!active && ctx->all_active) {  // the step now follows the active list
        ctx->all_active = false;
        ctx->graph_dirty = true;
    }
    return KZG_OK;
}

kzg_status kzg_edit_bodies(kzg_ctx* k, const kzg_body_edit* edits, uint32_t n) {
    if (check(k) || (n && !edits)) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    for (uint32_t i = 0; i < n; ++i)
        if (edits[i].op > KZG_EDIT_DEACTIVATE) {
            ctx->err = "kzg_edit_bodies: edit " + std::to_string(i) + " has an unknown op";
            return KZG_ERR_INVALID;
        }
    if (n == 0) return KZG_OK;
    CK(cudaSetDevice(ctx->device));
    SETTLE(ctx);
    kzg_status s = finalize_bodies(k);
    if (s != KZG_OK) return s;
    kzg_body_edit* dev = nullptr;
    CK(cudaMalloc((void**)&dev, sizeof(kzg_body_edit) * n));
    cudaError_t e = cudaMemcpyAsync(dev, edits, sizeof(kzg_body_edit) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = edit_bodies(*ctx, dev, n);
    cudaFree(dev);
    CK(e);
    for (uint32_t i = 0; i < n && ctx->all_active; ++i)
        if (edits[i].op == KZG_EDIT_DEACTIVATE) {  // the step now follows the active list
            ctx->all_active = false;
            ctx->graph_dirty = true;
        }
    return KZG_OK;
}

kzg_status kzg_get_active_bodies(kzg_ctx* k, uint32_t* packed_ids, uint32_t capacity, uint32_t* count) {
    if (check(k) || !count) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    CK(cudaSetDevice(ctx->device));
    uint32_t n = 0;
    CK(cudaMemcpyAsync(&n, &ctx->dcnt->nact, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    *count = n;
    if (!packed_ids || capacity == 0 || n == 0) return KZG_OK;
    const uint32_t m = std::min(n, capacity);
    std::vector<uint32_t> slots(m), packed(ctx->nbodies);
    CK(cudaMemcpy(slots.data(), ctx->alist, sizeof(uint32_t) * m, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(packed.data(), ctx->b.packed, sizeof(uint32_t) * ctx->nbodies, cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < m; ++i) packed_ids[i] = packed[slots[i]];
    return KZG_OK;
}

kzg_status kzg_state_hash(kzg_ctx* k, uint64_t* out) {
    if (check(k) || !out) return KZG_ERR_INVALID;
    return hash_state(k->c, out);
}

kzg_status kzg_get_stats(kzg_ctx* k, kzg_stats* out) {
    if (check(k) || !out) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    if (ctx->sleep_count_pending) {
        CK(cudaSetDevice(ctx->device));
        SETTLE(ctx);
    }
    *out = ctx->stats;
    out->cache_capacity = k->c.cache_cap;  // the table as it is now (it may have grown since)
    return KZG_OK;
}

kzg_status kzg_num_pairs(kzg_ctx* k, uint32_t* n) {
    if (check(k) || !n) return KZG_ERR_INVALID;
    *n = k->c.hcnt->npairs;
    return KZG_OK;
}

kzg_status kzg_download_pairs(kzg_ctx* k, uint32_t* out, uint32_t cap) {
    if (check(k) || !out) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    uint32_t n = std::min(ctx->hcnt->npairs, cap);
    std::vector<uint2> p(n);
    std::vector<uint32_t> packed(ctx->nbodies);
    if (n) CK(cudaMemcpy(p.data(), ctx->pairs, sizeof(uint2) * n, cudaMemcpyDeviceToHost));
    if (ctx->nbodies) CK(cudaMemcpy(packed.data(), ctx->b.packed, 4 * ctx->nbodies, cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < n; ++i) {
        out[2 * i] = p[i].x == 0xFFFFFFFFu ? 0xFFFFFFFFu : packed[p[i].x];
        out[2 * i + 1] = p[i].y == 0xFFFFFFFFu ? 0xFFFFFFFFu : packed[p[i].y];
    }
    return KZG_OK;
}

kzg_status kzg_num_constraints(kzg_ctx* k, uint32_t* n) {
    if (check(k) || !n) return KZG_ERR_INVALID;
    *n = k->c.hcnt->ncons;
    return KZG_OK;
}

kzg_status kzg_download_constraints(kzg_ctx* k, uint32_t* hdr, float* fr, float* pts, uint32_t cap) {
    if (check(k)) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    const uint32_t n = std::min(ctx->hcnt->ncons, cap);
    if (!n) return KZG_OK;
    std::vector<uint32_t> a(n), b(n), np(n);
    std::vector<float2> f(n);
    CK(cudaMemcpy(a.data(), ctx->con_a, 4 * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(b.data(), ctx->con_b, 4 * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(np.data(), ctx->con_np, 4 * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(f.data(), ctx->con_fr, sizeof(float2) * n, cudaMemcpyDeviceToHost));
    const size_t R = 4ull * n;
    const DeviceRows& r = ctx->r;
    std::vector<float4> pA(R), pB(R), nn(R), t1(R), t2(R), rA(R), rB(R), laA(R), laB(R), m(R), im(R), bi(R);
    float4* srcs[] = {r.pA, r.pB, r.n, r.t1, r.t2, r.rA, r.rB, r.laA, r.laB, r.mass, r.imp, r.bias};
    std::vector<float4>* dsts[] = {&pA, &pB, &nn, &t1, &t2, &rA, &rB, &laA, &laB, &m, &im, &bi};
    for (int q = 0; q < 12; ++q) CK(cudaMemcpy(dsts[q]->data(), srcs[q], sizeof(float4) * R, cudaMemcpyDeviceToHost));
    std::vector<uint32_t> packed(ctx->nbodies);
    CK(cudaMemcpy(packed.data(), ctx->b.packed, 4 * ctx->nbodies, cudaMemcpyDeviceToHost));
    for (uint32_t c = 0; c < n; ++c) {
        if (hdr) { hdr[3 * c] = packed[a[c]]; hdr[3 * c + 1] = packed[b[c]]; hdr[3 * c + 2] = np[c]; }
        if (fr) { fr[2 * c] = f[c].x; fr[2 * c + 1] = f[c].y; }
        if (!pts) continue;
        for (uint32_t p = 0; p < 8; ++p) {
            float* o = pts + (8ull * c + p) * 39;
            std::memset(o, 0, sizeof(float) * 39);
            if (p >= np[c]) continue;
            size_t j = 4ull * c + p;
            auto put = [&](int at, const float4& v) { o[at] = v.x; o[at + 1] = v.y; o[at + 2] = v.z; };
            put(0, pA[j]); put(3, pB[j]); put(6, nn[j]); o[9] = pA[j].w;
            std::memcpy(&o[10], &pB[j].w, 4);
            put(11, rA[j]); put(14, rB[j]); put(17, laA[j]); put(20, laB[j]); put(23, t1[j]); put(26, t2[j]);
            o[29] = m[j].x; o[30] = m[j].y; o[31] = m[j].z;
            o[32] = im[j].x; o[33] = im[j].y; o[34] = im[j].z;
            o[35] = bi[j].x; o[36] = bi[j].y; o[37] = im[j].w; o[38] = bi[j].z;
        }
    }
    return KZG_OK;
}

// ---- device snapshots: body state, the manifold cache and the joints, for exact resume -------
namespace {
constexpr uint32_t kSnapMagic = 0x53475A4Bu;  // 'KZGS'
constexpr uint32_t kSnapVersion = 4;
struct SnapHeader {
    uint32_t magic, version, nbodies, cache_cap, cache_entries, cache_used, njoints, reserved;  // reserved: active-list length
};
constexpr int kSnapBodyArrays = 10;  // pos, rot, lv, av, plv, pav, force, torque, fat bounds (+ 3 iiw columns)
// + per body: activity, sleep timer, island index, active-list position, active-list buffer entry
constexpr size_t kSnapBodyBytes = sizeof(float4) * (kSnapBodyArrays + 3) + 5 * sizeof(uint32_t);
constexpr size_t kSnapCacheBytes = sizeof(uint32_t) + sizeof(unsigned long long) + sizeof(uint32_t) + 8 * sizeof(float4);

float4** snap_body_arrays(DeviceBodies& b, float4** out) {
    float4* a[kSnapBodyArrays] = {b.pos, b.rot, b.lv, b.av, b.plv, b.pav, b.force, b.torque, b.fat_mn, b.fat_mx};
    for (int i = 0; i < kSnapBodyArrays; ++i) out[i] = a[i];
    return out;
}
}  // namespace

kzg_status kzg_snapshot_size(kzg_ctx* k, size_t* bytes) {
    if (check(k) || !bytes) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    const size_t H = ctx->cache_cap;
    std::vector<unsigned long long> keys(H);
    CK(cudaMemcpy(keys.data(), ctx->c_key, sizeof(unsigned long long) * H, cudaMemcpyDeviceToHost));
    size_t used = 0;
    for (unsigned long long key : keys) used += key != 0ull;
    *bytes = sizeof(SnapHeader) + kSnapBodyBytes * ctx->nbodies + kSnapCacheBytes * used +
             joint_record_bytes() * ctx->njoints;
    return KZG_OK;
}

kzg_status kzg_snapshot_save(kzg_ctx* k, void* out, size_t capacity) {
    if (check(k) || !out) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    const size_t H = ctx->cache_cap, nb = ctx->nbodies;
    std::vector<unsigned long long> keys(H);
    std::vector<uint32_t> np(H);
    std::vector<float4> pos(4 * H), imp(4 * H);
    CK(cudaMemcpy(keys.data(), ctx->c_key, sizeof(unsigned long long) * H, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(np.data(), ctx->c_np, sizeof(uint32_t) * H, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(pos.data(), ctx->c_pos, sizeof(float4) * 4 * H, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(imp.data(), ctx->c_imp, sizeof(float4) * 4 * H, cudaMemcpyDeviceToHost));
    size_t used = 0;
    for (unsigned long long key : keys) used += key != 0ull;
    const size_t JB = joint_record_bytes() * ctx->njoints;
    const size_t need = sizeof(SnapHeader) + kSnapBodyBytes * nb + kSnapCacheBytes * used + JB;
    if (capacity < need) {
        ctx->err = "kzg_snapshot_save: buffer smaller than kzg_snapshot_size";
        return KZG_ERR_CAPACITY;
    }
    uint8_t* p = static_cast<uint8_t*>(out);
    SnapHeader h{kSnapMagic, kSnapVersion, (uint32_t)nb, (uint32_t)H, ctx->hcnt->cache_entries, (uint32_t)used,
                 ctx->njoints, 0u};
    CK(cudaMemcpy(&h.cache_entries, &ctx->dcnt->cache_entries, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    std::memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    float4* arrs[kSnapBodyArrays];
    snap_body_arrays(ctx->b, arrs);
    for (int a = 0; a < kSnapBodyArrays; ++a) {
        CK(cudaMemcpy(p, arrs[a], sizeof(float4) * nb, cudaMemcpyDeviceToHost));
        p += sizeof(float4) * nb;
    }
    CK(cudaMemcpy(p, ctx->b.iiw, sizeof(float4) * 3 * nb, cudaMemcpyDeviceToHost));
    p += sizeof(float4) * 3 * nb;
    for (void* a : {(void*)ctx->b.act, (void*)ctx->b.sleep_t, (void*)ctx->b.isl_idx, (void*)ctx->b.apos, (void*)ctx->alist}) {
        CK(cudaMemcpy(p, a, sizeof(uint32_t) * nb, cudaMemcpyDeviceToHost));
        p += sizeof(uint32_t) * nb;
    }
    CK(cudaMemcpy(&h.reserved, &ctx->dcnt->nact, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    std::memcpy(out, &h, sizeof(h));  // header again with the active-list length
    for (size_t slot = 0; slot < H; ++slot) {  // occupied slots of the open-addressing table
        if (!keys[slot]) continue;
        const uint32_t s32 = (uint32_t)slot;
        std::memcpy(p, &s32, 4); p += 4;
        std::memcpy(p, &keys[slot], 8); p += 8;
        std::memcpy(p, &np[slot], 4); p += 4;
        std::memcpy(p, &pos[4 * slot], 4 * sizeof(float4)); p += 4 * sizeof(float4);
        std::memcpy(p, &imp[4 * slot], 4 * sizeof(float4)); p += 4 * sizeof(float4);
    }
    if (JB) CK(cudaMemcpy(p, ctx->joints, JB, cudaMemcpyDeviceToHost));
    return KZG_OK;
}

kzg_status kzg_snapshot_load(kzg_ctx* k, const void* in, size_t size) {
    if (check(k) || !in || size < sizeof(SnapHeader)) return KZG_ERR_INVALID;
    Ctx* ctx = &k->c;
    CK(cudaSetDevice(ctx->device));
    SETTLE(ctx);
    kzg_status st = finalize_bodies(k);
    if (st != KZG_OK) return st;
    SnapHeader h;
    std::memcpy(&h, in, sizeof(h));
    const size_t nb = ctx->nbodies, H = h.cache_cap;  // the table takes the snapshot's capacity
    const size_t JB = joint_record_bytes() * ctx->njoints;
    if (h.magic != kSnapMagic || h.version != kSnapVersion || h.nbodies != nb || h.cache_cap == 0 ||
        (h.cache_cap & (h.cache_cap - 1u)) != 0 || h.cache_used > h.cache_cap || h.cache_entries > h.cache_cap ||
        h.njoints != ctx->njoints ||
        size != sizeof(SnapHeader) + kSnapBodyBytes * nb + kSnapCacheBytes * (size_t)h.cache_used + JB) {
        ctx->err = "kzg_snapshot_load: snapshot does not match this context (bodies, joints, cache table or size)";
        return KZG_ERR_INVALID;
    }
    {  // every cache slot inside the table, checked before anything is written
        const uint8_t* q = static_cast<const uint8_t*>(in) + sizeof(h) + kSnapBodyBytes * nb;
        for (uint32_t e = 0; e < h.cache_used; ++e, q += kSnapCacheBytes) {
            uint32_t slot;
            std::memcpy(&slot, q, 4);
            if (slot >= H) {
                ctx->err = "kzg_snapshot_load: cache slot out of range";
                return KZG_ERR_INVALID;
            }
        }
    }
    CK(cudaStreamSynchronize(ctx->stream));
    const uint8_t* p = static_cast<const uint8_t*>(in) + sizeof(h);
    float4* arrs[kSnapBodyArrays];
    snap_body_arrays(ctx->b, arrs);
    for (int a = 0; a < kSnapBodyArrays; ++a) {
        CK(cudaMemcpy(arrs[a], p, sizeof(float4) * nb, cudaMemcpyHostToDevice));
        p += sizeof(float4) * nb;
    }
    CK(cudaMemcpy(ctx->b.iiw, p, sizeof(float4) * 3 * nb, cudaMemcpyHostToDevice));
    p += sizeof(float4) * 3 * nb;
    for (void* a : {(void*)ctx->b.act, (void*)ctx->b.sleep_t, (void*)ctx->b.isl_idx, (void*)ctx->b.apos, (void*)ctx->alist}) {
        CK(cudaMemcpy(a, p, sizeof(uint32_t) * nb, cudaMemcpyHostToDevice));
        p += sizeof(uint32_t) * nb;
    }
    if (h.reserved > nb) { ctx->err = "kzg_snapshot_load: active-list length out of range"; return KZG_ERR_INVALID; }
    CK(cudaMemcpy(&ctx->dcnt->nact, &h.reserved, sizeof(uint32_t), cudaMemcpyHostToDevice));
    ctx->all_active = h.reserved == nb;
    ctx->graph_dirty = true;
    const size_t used = h.cache_used;
    std::vector<uint32_t> slots(used), np(used);
    std::vector<unsigned long long> keys(used);
    std::vector<float4> pos(4 * used), imp(4 * used);
    for (size_t e = 0; e < used; ++e) {
        std::memcpy(&slots[e], p, 4); p += 4;
        std::memcpy(&keys[e], p, 8); p += 8;
        std::memcpy(&np[e], p, 4); p += 4;
        std::memcpy(&pos[4 * e], p, 4 * sizeof(float4)); p += 4 * sizeof(float4);
        std::memcpy(&imp[4 * e], p, 4 * sizeof(float4)); p += 4 * sizeof(float4);
    }
    st = cache_reset(*ctx, (uint32_t)H);
    if (st != KZG_OK) return st;
    st = cache_scatter(*ctx, slots.data(), keys.data(), np.data(), pos.data(), imp.data(), (uint32_t)used);
    if (st != KZG_OK) return st;
    CK(cudaMemcpy(&ctx->dcnt->cache_entries, &h.cache_entries, sizeof(uint32_t), cudaMemcpyHostToDevice));
    if (JB) CK(cudaMemcpy(ctx->joints, p, JB, cudaMemcpyHostToDevice));
    return KZG_OK;
}

kzg_status kzg_mlp_set_params(kzg_ctx* k, const float* theta, const float* mean, const float* stdv) {
    if (k) k->c.graph_dirty = true;
    if (check(k) || !theta || !mean || !stdv) return KZG_ERR_INVALID;
    return mlp_set_params(k->c, theta, mean, stdv);
}

kzg_status kzg_mlp_get_params(kzg_ctx* k, float* theta, float* mean, float* stdv) {
    if (check(k) || !theta) return KZG_ERR_INVALID;
    return mlp_get_params(k->c, theta, mean, stdv);
}

kzg_status kzg_mlp_enable(kzg_ctx* k, int enabled) {
    if (k) k->c.graph_dirty = true;
    if (check(k)) return KZG_ERR_INVALID;
    if (enabled && !k->c.mlp.have) {
        k->c.err = "kzg_mlp_enable: set the model parameters first";
        return KZG_ERR_INVALID;
    }
    k->c.mlp.enabled = enabled != 0;
    return KZG_OK;
}

kzg_status kzg_mlp_set_blend(kzg_ctx* k, float normal, float tangent) {
    if (k) k->c.graph_dirty = true;
    if (check(k) || !(normal >= 0.0f && normal <= 1.0f) || !(tangent >= 0.0f && tangent <= 1.0f))
        return KZG_ERR_INVALID;
    k->c.mlp.blend_n = normal;
    k->c.mlp.blend_t = tangent;
    return KZG_OK;
}

kzg_status kzg_mlp_set_quantile(kzg_ctx* k, float tau) {
    if (check(k) || !(tau >= 0.0f && tau < 1.0f)) return KZG_ERR_INVALID;
    k->c.mlp.tau = tau;
    return KZG_OK;
}

kzg_status kzg_mlp_log_begin(kzg_ctx* k, uint32_t capacity) {
    if (k) k->c.graph_dirty = true;
    if (check(k)) return KZG_ERR_INVALID;
    return mlp_log_begin(k->c, capacity);
}

kzg_status kzg_mlp_log_fetch(kzg_ctx* k, float* out, uint32_t capacity, uint32_t* count) {
    if (check(k) || !count) return KZG_ERR_INVALID;
    return mlp_log_fetch(k->c, out, capacity, count);
}

kzg_status kzg_mlp_set_dataset(kzg_ctx* k, const float* samples, uint32_t n) {
    if (check(k) || (n && !samples)) return KZG_ERR_INVALID;
    return mlp_set_dataset(k->c, samples, n);
}

kzg_status kzg_mlp_gradient(kzg_ctx* k, uint32_t first, uint32_t count, float* grad, float* loss) {
    if (check(k) || !grad) return KZG_ERR_INVALID;
    return mlp_gradient(k->c, first, count, grad, loss);
}

kzg_status kzg_mlp_train_step(kzg_ctx* k, uint32_t first, uint32_t count, float lr, float* loss) {
    if (check(k) || !(lr > 0.0f)) return KZG_ERR_INVALID;
    return mlp_train_step(k->c, first, count, lr, loss);
}

kzg_status kzg_mlp_predict(kzg_ctx* k, uint32_t first, uint32_t count, float* out) {
    if (check(k) || (count && !out)) return KZG_ERR_INVALID;
    return mlp_predict(k->c, first, count, out);
}

kzg_status kzg_hull_build(const float* pts, uint32_t n, uint32_t max_points, float* ov, uint32_t* onv, uint8_t* osz,
                          uint32_t* onf, uint32_t* oidx, uint32_t* oni, uint32_t cap_faces) {
    if (!pts || !ov || !onv || !osz || !onf || !oidx || !oni) return KZG_ERR_INVALID;
    int r = hull_build(pts, n, max_points ? max_points : 256, ov, onv, osz, onf, oidx, oni, cap_faces);
    if (r == -2) return KZG_ERR_CAPACITY;
    return r == 0 ? KZG_OK : KZG_ERR_INVALID;
}

kzg_status kzg_mass_properties(const kzg_shape_desc* shape, const float* hv, const uint8_t* fs, const uint32_t* fi,
                               uint32_t motion, float density, float mass_override, float* out_inv_mass,
                               float* out_iil) {
    if (!shape || !out_inv_mass || !out_iil) return KZG_ERR_INVALID;
    if (shape->type == KZG_SHAPE_HULL && (!hv || !fs || !fi)) return KZG_ERR_INVALID;
    mass_properties(*shape, hv, fs, fi, motion, density, mass_override, out_inv_mass, out_iil);
    return KZG_OK;
}

}  // extern "C"
