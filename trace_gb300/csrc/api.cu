// C ABI of libgbtrace: contexts, scenes, BVH lifetime, export and queries.
#include <cuda_runtime.h>

#include <cerrno>
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "gbt_internal.cuh"

// ---------------------------------------------------------------------------
// errors and scratch
// ---------------------------------------------------------------------------
int gbt_fail(gbt_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int gbt_cuda_fail(gbt_ctx *ctx, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return gbt_fail(ctx, e == cudaErrorMemoryAllocation ? GBT_ENOMEM : GBT_ECUDA, m);
}

int gbt_check_device_error(gbt_ctx *ctx, const char *what) {
    unsigned int flags = 0;
    GBT_CUDA(ctx, cudaMemcpyAsync(&flags, ctx->d_error, sizeof(flags), cudaMemcpyDeviceToHost, ctx->stream));
    GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (flags == 0) return GBT_OK;
    GBT_CUDA(ctx, cudaMemsetAsync(ctx->d_error, 0, sizeof(unsigned int), ctx->stream));
    GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    std::string m = std::string(what) + ": device reported";
    if (flags & GBT_DEVERR_SPIN) m += " [bounded wait ran out]";
    if (flags & GBT_DEVERR_BOUNDS) m += " [index out of range]";
    if (flags & GBT_DEVERR_STACK) m += " [traversal stack overflow]";
    if (flags & GBT_DEVERR_CAPACITY) m += " [work list full]";
    return gbt_fail(ctx, (flags & GBT_DEVERR_SPIN) ? GBT_ETIMEOUT : GBT_EDEVICE, m);
}

cudaError_t gbt_block_get(gbt_ctx *ctx, size_t bytes, void **p, size_t *got) {
    int best = -1;
    for (int i = 0; i < GBT_BLOCK_CACHE; i++) {
        const size_t b = ctx->block_cache_bytes[i];
        if (ctx->block_cache[i] && b >= bytes && b / 2 <= bytes && (best < 0 || b < ctx->block_cache_bytes[best]))
            best = i;
    }
    if (best >= 0) {
        *p = ctx->block_cache[best];
        *got = ctx->block_cache_bytes[best];
        ctx->block_cache[best] = nullptr;
        ctx->block_cache_bytes[best] = 0;
        return cudaSuccess;
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {  // room held by the cache may be what is missing
        cudaGetLastError();
        gbt_block_release(ctx);
        e = cudaMalloc(p, bytes);
    }
    *got = e == cudaSuccess ? bytes : 0;
    return e;
}

void gbt_block_put(gbt_ctx *ctx, void *p, size_t bytes) {
    if (!p) return;
    if (!ctx->keep_workspace || bytes == 0) {
        cudaFree(p);
        return;
    }
    int slot = -1;
    for (int i = 0; i < GBT_BLOCK_CACHE && slot < 0; i++)
        if (!ctx->block_cache[i]) slot = i;
    if (slot < 0) {
        slot = 0;
        for (int i = 1; i < GBT_BLOCK_CACHE; i++)
            if (ctx->block_cache_bytes[i] < ctx->block_cache_bytes[slot]) slot = i;
        if (ctx->block_cache_bytes[slot] >= bytes) {  // every cached block is larger: keep them
            cudaFree(p);
            return;
        }
        cudaFree(ctx->block_cache[slot]);
    }
    ctx->block_cache[slot] = p;
    ctx->block_cache_bytes[slot] = bytes;
}

void gbt_block_release(gbt_ctx *ctx) {
    for (int i = 0; i < GBT_BLOCK_CACHE; i++) {
        if (ctx->block_cache[i]) cudaFree(ctx->block_cache[i]);
        ctx->block_cache[i] = nullptr;
        ctx->block_cache_bytes[i] = 0;
    }
}

void *gbt_pinned(gbt_ctx *ctx) {
    if (!ctx->h_pin && cudaMallocHost(&ctx->h_pin, GBT_PINNED_BYTES) != cudaSuccess) {
        cudaGetLastError();
        ctx->h_pin = nullptr;
    }
    return ctx->h_pin;
}

int gbt_scratch(gbt_ctx *ctx, size_t bytes, void **out) {
    if (ctx->scratch_bytes < bytes) {
        if (ctx->scratch_pins > 0)
            return gbt_fail(ctx, GBT_EINVAL, "scratch: a live graph's rebuilds use the context's scratch, which "
                                             "cannot grow until the graph is destroyed");
        if (ctx->scratch) {
            GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            cudaFree(ctx->scratch);
        }
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
        size_t b = bytes + bytes / 4;
        if (cudaMalloc(&ctx->scratch, b) != cudaSuccess) {
            cudaGetLastError();
            return gbt_fail(ctx, GBT_ENOMEM, "scratch allocation of " + std::to_string(b) + " bytes");
        }
        ctx->scratch_bytes = b;
    }
    *out = ctx->scratch;
    return GBT_OK;
}

template <class T>
static int dalloc(gbt_ctx *ctx, T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), count * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return gbt_fail(ctx, GBT_ENOMEM, "device allocation of " + std::to_string(count * sizeof(T)) + " bytes");
    }
    return GBT_OK;
}

#define GBT_TRY(x)             \
    do {                       \
        int rc_ = (x);         \
        if (rc_) return rc_;   \
    } while (0)

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
extern "C" int gbt_ctx_create(int device, gbt_ctx **out) {
    if (!out) return GBT_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return GBT_ECUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess) return GBT_ECUDA;
    gbt_ctx *c = new gbt_ctx();
    c->device = device;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c->d_error, sizeof(unsigned int)) != cudaSuccess ||
        cudaMemset(c->d_error, 0, sizeof(unsigned int)) != cudaSuccess ||
        cudaMalloc(&c->d_counters, 4 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemset(c->d_counters, 0, 4 * sizeof(unsigned long long)) != cudaSuccess) {
        delete c;
        return GBT_ECUDA;
    }
    for (auto &e : c->ev) cudaEventCreate(&e);
    for (auto &e : c->tune_ev) cudaEventCreate(&e);
    if (const char *t = std::getenv("GBT_TRAVERSAL"))
        c->traversal = std::strcmp(t, "simple") == 0 ? 1 : std::strcmp(t, "ww") == 0 ? 2 : 0;
    if (const char *t = std::getenv("GBT_ANYHIT_LAST")) c->anyhit_last = std::strcmp(t, "0") != 0;
    if (const char *t = std::getenv("GBT_PRIMARY_TILES")) c->primary_tiles = std::strcmp(t, "0") != 0;
    if (const char *t = std::getenv("GBT_PRIMARY_PACKETS")) c->primary_packets = std::atoi(t) < 0 ? 0 : std::atoi(t) > 2 ? 2 : std::atoi(t);
    if (const char *t = std::getenv("GBT_SORT_THREADS")) c->sort_threads = std::atoi(t) == 512 ? 512 : 256;
    *out = c;
    return GBT_OK;
}

extern "C" int gbt_ctx_destroy(gbt_ctx *ctx) {
    if (!ctx) return GBT_EINVAL;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->rstate) cudaFree(ctx->rstate);
    if (ctx->d_error) cudaFree(ctx->d_error);
    if (ctx->d_counters) cudaFree(ctx->d_counters);
    if (ctx->d_out) cudaFree(ctx->d_out);
    if (ctx->bstate) cudaFree(ctx->bstate);
    gbt_phr_release(ctx);
    gbt_block_release(ctx);
    if (ctx->h_pin) cudaFreeHost(ctx->h_pin);
    for (auto &e : ctx->prof_ev) cudaEventDestroy(e);
    for (auto &e : ctx->ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : ctx->tune_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    delete ctx;
    return GBT_OK;
}

extern "C" const char *gbt_last_error(const gbt_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }
extern "C" void *gbt_ctx_stream(gbt_ctx *ctx) { return ctx ? static_cast<void *>(ctx->stream) : nullptr; }

extern "C" int gbt_ctx_set_profiling(gbt_ctx *ctx, int32_t level) {
    if (!ctx || level < 0 || level > 2) return GBT_EINVAL;
    if (level >= 1 && ctx->prof_ev.empty()) {
        ctx->prof_ev.resize(1024);
        for (auto &e : ctx->prof_ev) GBT_CUDA(ctx, cudaEventCreate(&e));
    }
    ctx->profiling = level;
    ctx->n_prof_ev = 0;
    return GBT_OK;
}

extern "C" int gbt_ctx_set_option(gbt_ctx *ctx, int32_t option, int32_t value) {
    if (!ctx) return GBT_EINVAL;
    switch (option) {
    case GBT_OPT_TRAVERSAL:
        if (value < 0 || value > 2) return gbt_fail(ctx, GBT_EINVAL, "set_option: traversal must be 0, 1 or 2");
        ctx->traversal = value;
        return GBT_OK;
    case GBT_OPT_ANYHIT_LAST:
    case GBT_OPT_PRIMARY_TILES:
        if (value < 0 || value > 1) return gbt_fail(ctx, GBT_EINVAL, "set_option: value must be 0 or 1");
        (option == GBT_OPT_ANYHIT_LAST ? ctx->anyhit_last : ctx->primary_tiles) = value;
        return GBT_OK;
    case GBT_OPT_PRIMARY_PACKETS:
        if (value < 0 || value > 2) return gbt_fail(ctx, GBT_EINVAL, "set_option: packets must be 0, 1 or 2");
        ctx->primary_packets = value;
        return GBT_OK;
    case GBT_OPT_PHR_SMALL_CUT:
        if (value < 1 || value > GBT_PHR_SMALL_CUT) return gbt_fail(ctx, GBT_EINVAL, "set_option: value must be 1..256");
        ctx->phr_small_cut = value;
        return GBT_OK;
    case GBT_OPT_KEEP_WORKSPACE:
        if (value < 0 || value > 1) return gbt_fail(ctx, GBT_EINVAL, "set_option: value must be 0 or 1");
        ctx->keep_workspace = value;
        if (!value) {
            GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            gbt_phr_release(ctx);
            gbt_block_release(ctx);
        }
        return GBT_OK;
    case GBT_OPT_SPIN_LIMIT:
        if (value < 1 || (uint32_t)value > GBT_SPIN_LIMIT)
            return gbt_fail(ctx, GBT_EINVAL, "set_option: spin limit must be 1..4194304");
        ctx->spin_limit = (uint32_t)value;
        return GBT_OK;
    case GBT_OPT_TEST_WITHHOLD_TILE:
        if (value < -1) return gbt_fail(ctx, GBT_EINVAL, "set_option: tile must be >= -1");
        ctx->withhold_tile = value < 0 ? 0xffffffffu : (uint32_t)value;
        return GBT_OK;
    case GBT_OPT_TEST_COLLAPSE_CAP:
        if (value < 0) return gbt_fail(ctx, GBT_EINVAL, "set_option: capacity must be >= 0");
        ctx->collapse_cap = (uint32_t)value;
        return GBT_OK;
    default:
        return gbt_fail(ctx, GBT_EINVAL, "set_option: unknown option " + std::to_string(option));
    }
}

void gbt_prof_begin(gbt_ctx *ctx) {
    if (ctx->profiling >= 1 && ctx->n_prof_ev + 2 <= (int)ctx->prof_ev.size())
        cudaEventRecord(ctx->prof_ev[ctx->n_prof_ev++], ctx->stream);
}

void gbt_prof_end(gbt_ctx *ctx) {
    if (ctx->profiling >= 1 && (ctx->n_prof_ev & 1))
        cudaEventRecord(ctx->prof_ev[ctx->n_prof_ev++], ctx->stream);
}

extern "C" int gbt_ctx_sync(gbt_ctx *ctx) {
    if (!ctx) return GBT_EINVAL;
    GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return gbt_check_device_error(ctx, "sync");
}

// ---------------------------------------------------------------------------
// scene
// ---------------------------------------------------------------------------
extern "C" int gbt_scene_upload(gbt_ctx *ctx, const float *verts, const float *normals, uint32_t n_tri,
                                const gbt_sphere *spheres, uint32_t n_sph, const uint32_t *prim_mat,
                                const gbt_material *mats, uint32_t n_mat, gbt_scene **out) {
    if (!ctx || !out) return GBT_EINVAL;
    *out = nullptr;
    if ((n_tri && !verts) || (n_sph && !spheres) || n_tri + n_sph == 0)
        return gbt_fail(ctx, GBT_EINVAL, "scene_upload: no primitives");
    if ((uint64_t)n_tri + n_sph >= (1ull << 30)) return gbt_fail(ctx, GBT_EINVAL, "scene_upload: too many primitives");
    const uint32_t n = n_tri + n_sph;
    std::vector<uint32_t> pm(n, 0);
    if (prim_mat) {
        for (uint32_t i = 0; i < n; i++) {
            if (prim_mat[i] >= (n_mat ? n_mat : 1))
                return gbt_fail(ctx, GBT_EINVAL, "scene_upload: material index out of range at primitive " + std::to_string(i));
            pm[i] = prim_mat[i];
        }
    }
    std::vector<gbt_material> mv;
    if (mats && n_mat) mv.assign(mats, mats + n_mat);
    else mv.push_back(gbt_material{GBT_MAT_DIFFUSE, {0.5f, 0.5f, 0.5f}, 0.f});
    // two float4 per material: (color.rgb, type), (param, 0, 0, 0)
    std::vector<float4> mf(2 * mv.size());
    for (size_t i = 0; i < mv.size(); i++) {
        if (mv[i].type < GBT_MAT_DIFFUSE || mv[i].type > GBT_MAT_REFRACTIVE)
            return gbt_fail(ctx, GBT_EINVAL, "scene_upload: unknown material type " + std::to_string(mv[i].type));
        if (mv[i].type == GBT_MAT_REFRACTIVE && !(mv[i].param > 0.f))
            return gbt_fail(ctx, GBT_EINVAL, "scene_upload: Refractive.Ratio must be > 0");
        float tf;
        std::memcpy(&tf, &mv[i].type, sizeof(tf));
        mf[2 * i] = make_float4(mv[i].color[0], mv[i].color[1], mv[i].color[2], tf);
        mf[2 * i + 1] = make_float4(mv[i].param, 0.f, 0.f, 0.f);
    }
    gbt_scene *s = new gbt_scene();
    s->ctx = ctx;
    s->n_tri = n_tri;
    s->n_sph = n_sph;
    s->n_mat = (uint32_t)mv.size();
    s->mats = mv;
    cudaStream_t st = ctx->stream;
    int rc = GBT_OK;
    if (!rc) rc = dalloc(ctx, &s->d_verts, (size_t)n_tri * 9);
    if (!rc && normals) rc = dalloc(ctx, &s->d_normals, (size_t)n_tri * 9);
    if (!rc) rc = dalloc(ctx, &s->d_sph, n_sph);
    if (!rc) rc = dalloc(ctx, &s->d_prim_mat, n);
    if (!rc) rc = dalloc(ctx, &s->d_mats, mf.size());
    if (rc) { gbt_scene_destroy(s); return rc; }
    cudaError_t e = cudaSuccess;
    if (n_tri) e = cudaMemcpyAsync(s->d_verts, verts, (size_t)n_tri * 9 * sizeof(float), cudaMemcpyHostToDevice, st);
    if (!e && normals) e = cudaMemcpyAsync(s->d_normals, normals, (size_t)n_tri * 9 * sizeof(float), cudaMemcpyHostToDevice, st);
    if (!e && n_sph) {
        std::vector<float4> sp(n_sph);
        for (uint32_t i = 0; i < n_sph; i++)
            sp[i] = make_float4(spheres[i].center[0], spheres[i].center[1], spheres[i].center[2], spheres[i].radius);
        e = cudaMemcpyAsync(s->d_sph, sp.data(), n_sph * sizeof(float4), cudaMemcpyHostToDevice, st);
        if (!e) e = cudaStreamSynchronize(st);
    }
    if (!e) e = cudaMemcpyAsync(s->d_prim_mat, pm.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(s->d_mats, mf.data(), mf.size() * sizeof(float4), cudaMemcpyHostToDevice, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) { gbt_scene_destroy(s); return gbt_cuda_fail(ctx, e, "scene_upload copy"); }
    *out = s;
    return GBT_OK;
}

extern "C" int gbt_scene_update_async(gbt_ctx *ctx, gbt_scene *scene, const float *d_verts) {
    if (!ctx || !scene || !d_verts) return GBT_EINVAL;
    GBT_CUDA(ctx, cudaMemcpyAsync(scene->d_verts, d_verts, (size_t)scene->n_tri * 9 * sizeof(float),
                                  cudaMemcpyDeviceToDevice, ctx->stream));
    return GBT_OK;
}

extern "C" int gbt_scene_destroy(gbt_scene *s) {
    if (!s) return GBT_EINVAL;
    if (s->ctx) cudaStreamSynchronize(s->ctx->stream);
    cudaFree(s->d_verts);
    cudaFree(s->d_normals);
    cudaFree(s->d_sph);
    cudaFree(s->d_prim_mat);
    cudaFree(s->d_mats);
    delete s;
    return GBT_OK;
}

// ---------------------------------------------------------------------------
// BVH lifetime
// ---------------------------------------------------------------------------
extern "C" int gbt_bvh_destroy(gbt_bvh *b) {
    if (!b) return GBT_EINVAL;
    if (b->ctx) cudaStreamSynchronize(b->ctx->stream);
    if (b->d_block) {
        if (b->ctx) gbt_block_put(b->ctx, b->d_block, b->d_block_bytes);
        else cudaFree(b->d_block);
        b->d_nodes = nullptr;
        b->d_prims = nullptr;
        b->d_hdr = nullptr;
        b->d_parent = nullptr;
    }
    if (b->d_nodes4 && b->ctx) {
        gbt_block_put(b->ctx, b->d_nodes4, b->nodes4_bytes);
        b->d_nodes4 = nullptr;
    }
    cudaFree(b->d_nodes);
    cudaFree(b->d_prims);
    cudaFree(b->d_hdr);
    cudaFree(b->d_codes);
    cudaFree(b->d_idx);
    cudaFree(b->d_run);
    cudaFree(b->d_ukey);
    cudaFree(b->d_parent);
    cudaFree(b->d_size);
    cudaFree(b->d_other);
    cudaFree(b->d_range);
    cudaFree(b->d_nodes4);
    cudaFree(b->d_hdr4);
    delete b;
    return GBT_OK;
}

static int lbvh_alloc(gbt_ctx *ctx, gbt_scene *sc, gbt_bvh **out) {
    const uint32_t n = sc->n_tri + sc->n_sph;
    gbt_bvh *b = new gbt_bvh();
    b->ctx = ctx;
    b->scene = sc;
    b->kind = GBT_BVH_LBVH;
    b->arity = 2;
    b->n_prim = n;
    b->node_cap = n > 1 ? n - 1 : 1;
    int rc = GBT_OK;
    if (!rc) rc = dalloc(ctx, &b->d_nodes, (size_t)b->node_cap * 4);
    if (!rc) rc = dalloc(ctx, &b->d_prims, (size_t)n * 3);
    if (!rc) rc = dalloc(ctx, &b->d_hdr, 1);
    if (!rc) rc = dalloc(ctx, &b->d_codes, (size_t)n * 2);
    if (!rc) rc = dalloc(ctx, &b->d_idx, (size_t)n * 2);
    if (!rc) rc = dalloc(ctx, &b->d_run, (size_t)n + 1);
    if (!rc) rc = dalloc(ctx, &b->d_ukey, n);
    if (!rc) rc = dalloc(ctx, &b->d_parent, n);
    if (!rc) rc = dalloc(ctx, &b->d_size, n);
    if (!rc) rc = dalloc(ctx, &b->d_other, n);
    if (!rc) rc = dalloc(ctx, &b->d_range, n);
    if (rc) { gbt_bvh_destroy(b); return rc; }
    *out = b;
    return GBT_OK;
}

extern "C" int gbt_lbvh_build(gbt_ctx *ctx, gbt_scene *scene, gbt_bvh **out) {
    if (!ctx || !scene || !out) return GBT_EINVAL;
    *out = nullptr;
    gbt_bvh *b = nullptr;
    GBT_TRY(lbvh_alloc(ctx, scene, &b));
    int rc = gbt_lbvh_enqueue(ctx, b);
    if (!rc) rc = gbt_check_device_error(ctx, "lbvh_build");
    if (!rc) rc = gbt_collapse4(ctx, b);
    if (!rc) rc = gbt_check_device_error(ctx, "lbvh_build traversal view");
    if (rc) { gbt_bvh_destroy(b); return rc; }
    *out = b;
    return GBT_OK;
}

extern "C" int gbt_lbvh_rebuild_async(gbt_ctx *ctx, gbt_bvh *bvh) {
    if (!ctx || !bvh || bvh->kind != GBT_BVH_LBVH) return gbt_fail(ctx, GBT_EINVAL, "rebuild: not an LBVH");
    bvh->has_nodes4 = 0;  // traversal uses the rebuilt binary nodes until gbt_bvh_set_layout(.., 4)
    bvh->packet_choice = 0;
    return gbt_lbvh_enqueue(ctx, bvh);
}

extern "C" int gbt_bvh_set_layout(gbt_ctx *ctx, gbt_bvh *bvh, int32_t width) {
    if (!ctx || !bvh || (width != 2 && width != 4)) return GBT_EINVAL;
    if (width == 2) {
        bvh->has_nodes4 = 0;
        bvh->packet_choice = 0;
        return GBT_OK;
    }
    GBT_TRY(gbt_collapse4(ctx, bvh));
    bvh->packet_choice = 0;
    return gbt_check_device_error(ctx, "bvh_set_layout");
}

extern "C" int gbt_bvh_set_packets(gbt_ctx *ctx, gbt_bvh *bvh, int32_t choice) {
    if (!ctx || !bvh || choice < 0 || choice > 2) return GBT_EINVAL;
    bvh->packet_choice = choice;
    return GBT_OK;
}

extern "C" int gbt_bvh_get_packets(gbt_ctx *ctx, gbt_bvh *bvh, int32_t *choice) {
    if (!ctx || !bvh || !choice) return GBT_EINVAL;
    *choice = bvh->packet_choice;
    return GBT_OK;
}

static int phr_build(gbt_ctx *ctx, gbt_bvh *aux, double alpha, double delta, int32_t branching, bool view,
                     gbt_bvh **out) {
    if (!ctx || !aux || !out) return GBT_EINVAL;
    *out = nullptr;
    if (aux->kind != GBT_BVH_LBVH) return gbt_fail(ctx, GBT_EINVAL, "phr_build: the auxiliary BVH must be an LBVH");
    if (branching < 2 || branching > 4) return gbt_fail(ctx, GBT_EUNSUPPORTED, "phr_build: branching factor must be 2..4");
    gbt_bvh *b = new gbt_bvh();
    b->ctx = ctx;
    b->scene = aux->scene;
    b->kind = GBT_BVH_PHR;
    b->arity = branching == 2 ? 2 : 4;
    int rc = gbt_phr_run(ctx, aux, alpha, delta, branching, b);
    if (!rc) rc = gbt_check_device_error(ctx, "phr_build");
    if (!rc && view) rc = gbt_collapse4(ctx, b);
    if (!rc && view) rc = gbt_check_device_error(ctx, "phr_build traversal view");
    if (rc) { gbt_bvh_destroy(b); return rc; }
    *out = b;
    return GBT_OK;
}

extern "C" int gbt_phr_build(gbt_ctx *ctx, gbt_bvh *aux, double alpha, double delta, int32_t branching, gbt_bvh **out) {
    return phr_build(ctx, aux, alpha, delta, branching, true, out);
}

extern "C" int gbt_phr_build_with_cost(gbt_ctx *ctx, gbt_bvh *aux, double alpha, double delta, int32_t branching,
                                       gbt_bvh **out, int64_t *build_cost) {
    if (!build_cost) return GBT_EINVAL;
    int rc = phr_build(ctx, aux, alpha, delta, branching, true, out);
    *build_cost = rc ? 0 : (*out)->build_cost;
    return rc;
}

// ---------------------------------------------------------------------------
// export (host-side depth-first walk of the downloaded nodes)
// ---------------------------------------------------------------------------
struct HostTree {
    BvhHeader hdr;
    int arity;
    std::vector<float4> nodes;
    std::vector<int32_t> rec_id;  // primitive id of each record
};

static int download_tree(gbt_ctx *ctx, gbt_bvh *b, HostTree &t) {
    GBT_CUDA(ctx, cudaMemcpyAsync(&t.hdr, b->d_hdr, sizeof(BvhHeader), cudaMemcpyDeviceToHost, ctx->stream));
    GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    t.arity = b->arity;
    size_t per = b->arity == 2 ? 4 : 8;
    t.nodes.resize((size_t)t.hdr.n_nodes * per + 1);
    if (t.hdr.n_nodes)
        GBT_CUDA(ctx, cudaMemcpyAsync(t.nodes.data(), b->d_nodes, (size_t)t.hdr.n_nodes * per * sizeof(float4),
                                      cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<float4> r0(b->n_prim);
    GBT_CUDA(ctx, cudaMemcpy2DAsync(r0.data(), sizeof(float4), b->d_prims, 3 * sizeof(float4), sizeof(float4), b->n_prim,
                                    cudaMemcpyDeviceToHost, ctx->stream));
    GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    t.rec_id.resize(b->n_prim);
    for (uint32_t i = 0; i < b->n_prim; i++) {
        int32_t v;
        std::memcpy(&v, &r0[i].w, 4);
        t.rec_id[i] = v;
    }
    return GBT_OK;
}

struct ChildRef {
    int32_t ref, cnt;
    float lo[3], hi[3];
};

static int children_of(const HostTree &t, int32_t node, ChildRef *out) {
    int k = 0;
    if (t.arity == 2) {
        const float4 *nd = &t.nodes[4 * (size_t)node];
        int32_t e[4];
        std::memcpy(e, &nd[3], 16);
        for (int c = 0; c < 2; c++) {
            if (e[2 * c + 1] < 0) continue;
            const float4 &xy = nd[c];
            const float *z = reinterpret_cast<const float *>(&nd[2]) + 2 * c;
            ChildRef r{e[2 * c], e[2 * c + 1], {xy.x, xy.z, z[0]}, {xy.y, xy.w, z[1]}};
            out[k++] = r;
        }
    } else {
        const float *m = reinterpret_cast<const float *>(&t.nodes[8 * (size_t)node]);
        int32_t ref[4], cnt[4];
        std::memcpy(ref, m + 24, 16);
        std::memcpy(cnt, m + 28, 16);
        for (int c = 0; c < 4; c++) {
            if (cnt[c] < 0) continue;
            ChildRef r{ref[c], cnt[c], {m[c], m[8 + c], m[16 + c]}, {m[4 + c], m[12 + c], m[20 + c]}};
            out[k++] = r;
        }
    }
    return k;
}

struct ExportOut {
    std::vector<int8_t> kind;
    std::vector<int32_t> count;
    std::vector<double> box;
    std::vector<int32_t> prims;
};

static void walk(const HostTree &t, ExportOut &o) {
    struct Item { ChildRef c; };
    std::vector<ChildRef> st;
    ChildRef root{t.hdr.root_ref, t.hdr.root_cnt, {t.hdr.root_lo[0], t.hdr.root_lo[1], t.hdr.root_lo[2]},
                  {t.hdr.root_hi[0], t.hdr.root_hi[1], t.hdr.root_hi[2]}};
    st.push_back(root);
    ChildRef ch[4];
    while (!st.empty()) {
        ChildRef c = st.back();
        st.pop_back();
        for (int k = 0; k < 3; k++) o.box.push_back(c.lo[k]);
        for (int k = 0; k < 3; k++) o.box.push_back(c.hi[k]);
        if (c.cnt > 0) {
            o.kind.push_back(1);
            o.count.push_back(c.cnt);
            for (int32_t s = c.ref; s < c.ref + c.cnt; s++) o.prims.push_back(t.rec_id[s]);
        } else {
            int k = children_of(t, c.ref, ch);
            o.kind.push_back(0);
            o.count.push_back(k);
            for (int j = k - 1; j >= 0; j--) st.push_back(ch[j]);
        }
    }
}

static int export_tree(gbt_ctx *ctx, gbt_bvh *b, ExportOut &o) {
    HostTree t;
    GBT_TRY(download_tree(ctx, b, t));
    walk(t, o);
    return GBT_OK;
}

extern "C" int gbt_bvh_counts(gbt_ctx *ctx, gbt_bvh *bvh, int64_t counts[4]) {
    if (!ctx || !bvh || !counts) return GBT_EINVAL;
    ExportOut o;
    GBT_TRY(export_tree(ctx, bvh, o));
    int64_t leaves = 0;
    for (auto k : o.kind) leaves += k;
    counts[0] = (int64_t)o.kind.size();
    counts[1] = leaves;
    counts[2] = (int64_t)o.prims.size();
    counts[3] = o.kind.empty() ? 0 : o.kind[0];
    return GBT_OK;
}

extern "C" int gbt_bvh_export(gbt_ctx *ctx, gbt_bvh *bvh, int8_t *kind, int32_t *count, double *box, int32_t *prims) {
    if (!ctx || !bvh) return GBT_EINVAL;
    ExportOut o;
    GBT_TRY(export_tree(ctx, bvh, o));
    if (kind) std::memcpy(kind, o.kind.data(), o.kind.size());
    if (count) std::memcpy(count, o.count.data(), o.count.size() * sizeof(int32_t));
    if (box) std::memcpy(box, o.box.data(), o.box.size() * sizeof(double));
    if (prims) std::memcpy(prims, o.prims.data(), o.prims.size() * sizeof(int32_t));
    return GBT_OK;
}

extern "C" int gbt_bvh_cost(gbt_ctx *ctx, gbt_bvh *bvh, double *cost) {
    if (!ctx || !bvh || !cost) return GBT_EINVAL;
    return gbt_cost_device(ctx, bvh, cost);  // bvh.go:226-239, evaluated on the device (cost.cu)
}

// gridOptimizer.OptimizedPHRparams (optimizer.go:44-84) with omega and evalPHR
// (optimizer.go:86-94): every (alpha, delta) of the grid, alphas outer, is built
// on the device with its build cost and its SAH cost (bvh.go:226-239, also on
// the device); the first minimum of the normalised score wins.
extern "C" int gbt_phr_optimize_grid(gbt_ctx *ctx, gbt_bvh *aux, int32_t branching, const double *alphas,
                                     int32_t n_alpha, const double *deltas, int32_t n_delta, int32_t frame_width,
                                     int32_t frame_height, double *alpha, double *delta, double *evals) {
    if (!ctx || !aux || !alphas || !deltas || !alpha || !delta) return GBT_EINVAL;
    if (n_alpha < 1 || n_delta < 1 || frame_width < 1 || frame_height < 1)
        return gbt_fail(ctx, GBT_EINVAL, "phr_optimize_grid: empty grid or frame");
    struct Eval { double sah; int64_t build; double a, d; };
    std::vector<Eval> ev;
    for (int32_t i = 0; i < n_alpha; i++) {
        for (int32_t j = 0; j < n_delta; j++) {
            gbt_bvh *b = nullptr;
            GBT_TRY(phr_build(ctx, aux, alphas[i], deltas[j], branching, false, &b));
            double sah = 0.0;
            int rc = gbt_bvh_cost(ctx, b, &sah);
            const int64_t bc = b->build_cost;
            gbt_bvh_destroy(b);
            if (rc) return rc;
            ev.push_back({sah, bc, alphas[i], deltas[j]});
        }
    }
    int64_t max_build = 0;
    double max_sah = 0.0;
    for (const Eval &e : ev) {
        if (e.build > max_build) max_build = e.build;
        if (e.sah > max_sah) max_sah = e.sah;
    }
    const double q = (double)aux->n_prim / 2000000.0;               // PRIM_THRESH
    const double o = (q * q) * ((double)frame_width * (double)frame_height / 200000.0);  // RES_THRESH
    double best = DBL_MAX;
    size_t bi = 0;
    for (size_t k = 0; k < ev.size(); k++) {
        const double c = (double)ev[k].build / (double)max_build + (o * o) * (ev[k].sah / max_sah);
        if (c < best) {
            best = c;
            bi = k;
        }
        if (evals) {
            evals[2 * k] = ev[k].sah;
            evals[2 * k + 1] = (double)ev[k].build;
        }
    }
    *alpha = ev[bi].a;
    *delta = ev[bi].d;
    return GBT_OK;
}

extern "C" int gbt_bvh_size(gbt_ctx *ctx, gbt_bvh *bvh, int64_t *size) {
    int64_t c[4];
    GBT_TRY(gbt_bvh_counts(ctx, bvh, c));
    *size = c[0];
    return GBT_OK;
}

extern "C" int gbt_lbvh_sorted(gbt_ctx *ctx, gbt_bvh *b, uint64_t *codes, int32_t *idx) {
    if (!ctx || !b || b->kind != GBT_BVH_LBVH) return gbt_fail(ctx, GBT_EINVAL, "lbvh_sorted: not an LBVH");
    BvhHeader h;
    GBT_CUDA(ctx, cudaMemcpyAsync(&h, b->d_hdr, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    size_t off = h.sorted_sel ? b->n_prim : 0;
    if (codes)
        GBT_CUDA(ctx, cudaMemcpyAsync(codes, b->d_codes + off, (size_t)b->n_prim * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (idx)
        GBT_CUDA(ctx, cudaMemcpyAsync(idx, b->d_idx + off, (size_t)b->n_prim * 4, cudaMemcpyDeviceToHost, ctx->stream));
    GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GBT_OK;
}

// ---------------------------------------------------------------------------
// queries
// ---------------------------------------------------------------------------
extern "C" int gbt_trace_async(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_ray *d_rays, uint32_t n, gbt_hit *d_hits) {
    if (!ctx || !bvh || (n && (!d_rays || !d_hits))) return GBT_EINVAL;
    return gbt_trace_enqueue(ctx, bvh, d_rays, n, d_hits);
}

extern "C" int gbt_trace(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_ray *rays, uint32_t n, gbt_hit *hits) {
    if (!ctx || !bvh || (n && (!rays || !hits))) return GBT_EINVAL;
    if (n == 0) return GBT_OK;
    gbt_ray *dr = nullptr;
    gbt_hit *dh = nullptr;
    GBT_TRY(dalloc(ctx, &dr, n));
    int rc = dalloc(ctx, &dh, n);
    cudaError_t e = cudaSuccess;
    if (!rc) e = cudaMemcpyAsync(dr, rays, (size_t)n * sizeof(gbt_ray), cudaMemcpyHostToDevice, ctx->stream);
    if (!rc && !e) rc = gbt_trace_enqueue(ctx, bvh, dr, n, dh);
    if (!rc && !e) e = cudaMemcpyAsync(hits, dh, (size_t)n * sizeof(gbt_hit), cudaMemcpyDeviceToHost, ctx->stream);
    if (!rc && !e) rc = gbt_check_device_error(ctx, "trace");
    cudaStreamSynchronize(ctx->stream);
    cudaFree(dr);
    cudaFree(dh);
    if (e) return gbt_cuda_fail(ctx, e, "trace copy");
    return rc;
}

extern "C" int gbt_render_async(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *p, float *d_rgb) {
    if (!ctx || !bvh || !cam || !p || !d_rgb) return GBT_EINVAL;
    return gbt_render_enqueue(ctx, bvh, cam, p, d_rgb);
}

extern "C" int gbt_render_last_stats(gbt_ctx *ctx, gbt_render_stats *stats) {
    if (!ctx || !stats) return GBT_EINVAL;
    unsigned long long c[4] = {0, 0, 0, 0};
    GBT_CUDA(ctx, cudaMemcpyAsync(c, ctx->d_counters, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream));
    GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double ms = 0.0;
    for (int i = 0; i + 1 < ctx->n_prof_ev; i += 2) {
        float m = 0.f;
        if (cudaEventElapsedTime(&m, ctx->prof_ev[i], ctx->prof_ev[i + 1]) == cudaSuccess) ms += m;
    }
    ctx->last_stats.nodes_visited = c[0];
    ctx->last_stats.prims_tested = c[1];
    ctx->last_stats.rays_traced = c[2];
    ctx->last_stats.ms_traverse = ms;
    *stats = ctx->last_stats;
    // stats accumulate from one read to the next
    ctx->last_stats = gbt_render_stats{};
    ctx->n_prof_ev = 0;
    GBT_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, 4 * sizeof(unsigned long long), ctx->stream));
    return GBT_OK;
}

extern "C" int gbt_render(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *p, float *rgb,
                          gbt_render_stats *stats) {
    if (!ctx || !bvh || !cam || !p || !rgb) return GBT_EINVAL;
    if (p->width < 2 || p->height < 2) return gbt_fail(ctx, GBT_EINVAL, "render: width and height must be >= 2");
    size_t bytes = (size_t)p->width * p->height * 3 * sizeof(float);
    // A page-locked host image (cudaMallocHost, cudaHostAlloc or cudaHostRegister)
    // is mapped into the device's address space: the last kernel of the frame
    // writes it directly, with no copy of the image afterwards.  Other host
    // memory receives the image by a copy from a device buffer.
    float *direct = nullptr;
    {
        cudaPointerAttributes pa;
        if (cudaPointerGetAttributes(&pa, rgb) == cudaSuccess) {
            if (pa.type == cudaMemoryTypeHost && pa.devicePointer) direct = static_cast<float *>(pa.devicePointer);
        } else {
            cudaGetLastError();
        }
    }
    if (!direct && ctx->d_out_bytes < bytes) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->d_out);
        ctx->d_out = nullptr;
        ctx->d_out_bytes = 0;
        GBT_TRY(dalloc(ctx, &ctx->d_out, bytes / sizeof(float)));
        ctx->d_out_bytes = bytes;
    }
    float *d = direct ? direct : ctx->d_out;
    cudaEventRecord(ctx->ev[0], ctx->stream);
    int rc = gbt_render_enqueue(ctx, bvh, cam, p, d);
    cudaEventRecord(ctx->ev[1], ctx->stream);
    cudaError_t e = cudaSuccess;
    if (!rc && !direct) e = cudaMemcpyAsync(rgb, d, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (!rc && !e) rc = gbt_check_device_error(ctx, "render");
    cudaStreamSynchronize(ctx->stream);
    if (e) return gbt_cuda_fail(ctx, e, "render copy");
    if (rc) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    ctx->last_stats.ms_total += ms;
    if (stats) return gbt_render_last_stats(ctx, stats);
    return GBT_OK;
}

// ---------------------------------------------------------------------------
// device memory helpers
// ---------------------------------------------------------------------------
extern "C" int gbt_device_alloc(gbt_ctx *ctx, size_t bytes, void **d_ptr) {
    if (!ctx || !d_ptr) return GBT_EINVAL;
    if (cudaMalloc(d_ptr, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        return gbt_fail(ctx, GBT_ENOMEM, "device_alloc");
    }
    return GBT_OK;
}
extern "C" int gbt_device_free(gbt_ctx *ctx, void *d_ptr) {
    if (!ctx) return GBT_EINVAL;
    cudaStreamSynchronize(ctx->stream);
    cudaFree(d_ptr);
    return GBT_OK;
}
extern "C" int gbt_host_alloc(gbt_ctx *ctx, size_t bytes, void **h_ptr) {
    if (!ctx || !h_ptr) return GBT_EINVAL;
    if (cudaMallocHost(h_ptr, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        return gbt_fail(ctx, GBT_ENOMEM, "host_alloc");
    }
    return GBT_OK;
}
extern "C" int gbt_host_free(gbt_ctx *ctx, void *h_ptr) {
    if (!ctx) return GBT_EINVAL;
    cudaFreeHost(h_ptr);
    return GBT_OK;
}
extern "C" int gbt_copy_h2d_async(gbt_ctx *ctx, void *d_dst, const void *h_src, size_t bytes) {
    if (!ctx) return GBT_EINVAL;
    GBT_CUDA(ctx, cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return GBT_OK;
}
extern "C" int gbt_copy_d2h_async(gbt_ctx *ctx, void *h_dst, const void *d_src, size_t bytes) {
    if (!ctx) return GBT_EINVAL;
    GBT_CUDA(ctx, cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return GBT_OK;
}

// ---------------------------------------------------------------------------
// OBJ loader (pkg/pt/obj.go:19-140)
// ---------------------------------------------------------------------------
static bool parse_int(const std::string &s, long &out) {
    if (s.empty()) return false;
    char *end = nullptr;
    errno = 0;
    long v = std::strtol(s.c_str(), &end, 10);
    if (errno || *end) return false;
    out = v;
    return true;
}

static bool parse_f(const std::string &s, double &out) {
    if (s.empty()) return false;
    char *end = nullptr;
    errno = 0;
    double v = std::strtod(s.c_str(), &end);
    if (*end) return false;
    out = v;
    return true;
}

extern "C" int gbt_obj_parse(const char *path, float *verts, float *normals, uint32_t *n_tri, int32_t *has_normals) {
    if (!path || !n_tri) return GBT_EINVAL;
    std::ifstream f(path);
    if (!f) return GBT_EINVAL;  // ParseFromPath panics on an open error (obj.go:12-14)
    // index 0 is a placeholder, so OBJ's 1-based indices index directly (obj.go:22-23)
    std::vector<double> V(3, 0.0), N(3, 0.0);
    const uint32_t cap = verts ? *n_tri : 0;  // on the filling call *n_tri is the buffer capacity
    uint32_t tris = 0;
    int32_t any_normals = 0;
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ls(line);
        std::vector<std::string> fields;
        std::string w;
        while (ls >> w) fields.push_back(w);
        if (fields.empty()) continue;
        const std::string &key = fields[0];
        if (key == "v" || key == "vn") {
            if (fields.size() < 4) return GBT_EINVAL;
            double x, y, z;
            for (size_t i = 1; i < fields.size(); i++)  // parseFloat validates every value (obj.go:130-140)
                if (!parse_f(fields[i], x)) return GBT_EINVAL;
            parse_f(fields[1], x);
            parse_f(fields[2], y);
            parse_f(fields[3], z);
            std::vector<double> &dst = key == "v" ? V : N;
            dst.push_back(x);
            dst.push_back(y);
            dst.push_back(z);
        } else if (key == "f") {
            std::vector<long> vi, ni;
            for (size_t a = 1; a < fields.size(); a++) {
                std::vector<std::string> parts;
                std::string cur;
                for (char c : fields[a]) {
                    if (c == '/') { parts.push_back(cur); cur.clear(); }
                    else cur.push_back(c);
                }
                parts.push_back(cur);
                long v;
                if (!parse_int(parts[0], v)) return GBT_EINVAL;
                if (v < 0) v = (long)(V.size() / 3) + v;  // negative index (obj.go:176-178)
                vi.push_back(v);
                if (parts.size() >= 3) {
                    long nn;
                    if (!parse_int(parts[2], nn)) return GBT_EINVAL;
                    if (nn < 0) nn = (long)(N.size() / 3) + nn;
                    ni.push_back(nn);
                }
            }
            bool with_n = ni.size() == fields.size() - 1;
            for (size_t i = 1; i + 2 <= vi.size(); i++) {  // fan triangulation (obj.go:193-203)
                long idx[3] = {vi[0], vi[i], vi[i + 1]};
                long nidx[3] = {with_n ? ni[0] : 0, with_n ? ni[i] : 0, with_n ? ni[i + 1] : 0};
                for (int k = 0; k < 3; k++) {
                    if (idx[k] < 0 || (size_t)idx[k] >= V.size() / 3) return GBT_EINVAL;
                    if (with_n && (nidx[k] < 0 || (size_t)nidx[k] >= N.size() / 3)) return GBT_EINVAL;
                }
                if (verts) {
                    if (tris >= cap) return GBT_EINVAL;
                    for (int k = 0; k < 3; k++)
                        for (int c = 0; c < 3; c++) verts[(size_t)tris * 9 + 3 * k + c] = (float)V[3 * idx[k] + c];
                    if (normals) {
                        for (int k = 0; k < 3; k++) {
                            if (with_n) {
                                for (int c = 0; c < 3; c++) normals[(size_t)tris * 9 + 3 * k + c] = (float)N[3 * nidx[k] + c];
                            } else {  // calcNormal per vertex (primitive.go:116-138)
                                const double *p0 = &V[3 * idx[k]], *p1 = &V[3 * idx[(k + 1) % 3]], *p2 = &V[3 * idx[(k + 2) % 3]];
                                double pa[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
                                double pb[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
                                double c3[3] = {pb[1] * pa[2] - pb[2] * pa[1], pb[2] * pa[0] - pb[0] * pa[2],
                                                pb[0] * pa[1] - pb[1] * pa[0]};
                                double l = std::sqrt(c3[0] * c3[0] + c3[1] * c3[1] + c3[2] * c3[2]);
                                for (int c = 0; c < 3; c++) normals[(size_t)tris * 9 + 3 * k + c] = (float)(c3[c] / l);
                            }
                        }
                    }
                }
                if (with_n) any_normals = 1;
                tris++;
            }
        }
    }
    *n_tri = tris;
    if (has_normals) *has_normals = any_normals;
    return GBT_OK;
}
