// insta_abi.cu -- host side of the C ABI: device residency of avatars (canonical mesh,
// per-frame BVHs, occupancy bitfields, field parameters), argument checking and launches.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include <cublas_v2.h>

#include "../../include/insta_gb300.h"
#include "device_common.cuh"
#include "mlp_tiles.cuh"
#include "kernels.h"

using namespace insta;

namespace {

struct Failure : std::runtime_error {
    int code;
    Failure(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw Failure(code, buf);
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) fail(INSTA_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

}  // namespace

struct Frame {
    DevBuf verts, frames, leaf_tris, nodes, bitfield;
    FrameView view{};
    bool has_occupancy = false;
    cudaEvent_t ready = nullptr;   // insta_frame_upload_async: recorded on the side stream
    bool pending = false;          // the main stream has not yet been made to wait for `ready`
};

struct Field {
    bool ready = false;
    insta_field_desc desc{};
    DevBuf params, image;
    TilePlan plan{};
    FieldView view{};
    uint64_t n_params = 0;
    // training: FP32 master weights (from the FP16 parameters at the first backward after a
    // load), Adam moments, the optimizer's step count and its FP16 output
    DevBuf w32, adam_m, adam_v, adam_steps, w16, ema;   // adam_steps: per hash-table entry
    // with an Ema the field's parameters are the average; the training weights' own FP16 copy,
    // weight image and view serve insta_field_eval_training
    DevBuf train_params, train_image, w16_train;
    FieldView train_view{};
    bool train_valid = false;
    bool w32_valid = false;
    uint32_t adam_step = 0;
    uint32_t ema_step = 0;   // steps averaged into `ema` (0: no running average yet)
};

// Device scratch of the render wavefront, sized for the largest request seen.
struct Wave {
    DevBuf rays[2][4], n_round, sample_index, sample_ray, sample_key, sample_order, sort_bins, samples, march_t, tiles, aux, out, out_f32,
        counters, req_table, req_meta, init_meta;
    uint32_t cap_rays = 0;
    uint64_t cap_samples = 0;
};

struct Avatar {
    int V = 0, F = 0;
    bool has_canon = false;
    DevBuf faces, mask, adjacency, canon_verts, canon_area, canon_frames;
    float render_min[3], render_max[3];
    float train_min[3] = {0.f, 0.f, 0.f}, train_max[3] = {1.f, 1.f, 1.f};
    uint32_t flags = 0;
    std::map<int, Frame> frames;
    DevBuf frame_table;
    bool table_dirty = true;
    uint32_t table_frames = 0;
    Field field;
    float center[3] = {0.f, 0.f, 0.f};   // TinyMesh::m_centorid of the canonical mesh (float sum / V)
    DevBuf density_grid;          // float [grid_cascades][128^3], Morton order (update_density_grid_nerf state)
    uint32_t grid_cascades = 0;
};

struct insta_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint64_t budget = 0, used = 0;
    std::map<int, std::unique_ptr<Avatar>> avatars;
    std::string last_error;
    uint32_t* err_dev = nullptr;
    uint32_t* ray_counter = nullptr;
    unsigned long long* sample_counter = nullptr;
    DevBuf out_rgba, out_depth, extra, bvh_scratch, frame_jobs, density_scratch, density_stage, side_scratch, map_scratch,
        grid_coords, grid_idx, grid_tmp;
    // the render loop as a CUDA graph (a conditional while node over pairs of rounds), rebuilt
    // when the wavefront's buffers or limits change
    cudaGraph_t loop_graph = nullptr;
    cudaGraphExec_t loop_exec = nullptr;
    std::vector<unsigned char> loop_key;
    uint32_t* loop_state = nullptr;                 // [0] steps of the current round, [1] rounds of this launch,
                                                    // [2] whether the body's second round ran
    unsigned long long* loop_rounds_total = nullptr; // rounds (low 40 bits) and loop iterations of graph launches
    unsigned long long loop_rounds_seen = 0;
    uint32_t loop_round_kernels = 10;                // kernels per graph-run round (9 with the fused field stage)
    unsigned long long* walk_stats = nullptr;        // nearest-walk counters while stage timing is on
    // insta_render_async with host outputs: double-buffered device staging, copied back on a
    // copy stream while the next render runs
    cudaStream_t copy = nullptr;
    cudaStream_t capture = nullptr;                 // captures the conditional second round of the graph body
    DevBuf async_rgba[2], async_depth[2];
    cudaEvent_t async_free[2] = {nullptr, nullptr}, async_done = nullptr;
    bool async_used[2] = {false, false};
    int async_next = 0;
    cublasHandle_t blas = nullptr;      // the training side's GEMMs
    bool train_tf32 = false;            // insta_train_set_math: TF32 tensor-core GEMMs
    bool train_tc = false;              // insta_train_set_math: the library's tcgen05 layer products
    DevBuf train_images;                // their weight images (rebuilt from the FP32 masters per call)
    DevBuf train_scratch;
    DevBuf loss_scratch;     // insta_train_loss: each kept ray's block start before compaction
    DevBuf train_t;          // insta_training_samples: each ray's sample positions t
    bool keep_master = false;           // a parameter reload from the optimizer keeps the FP32 master weights
    cudaStream_t side = nullptr;        // asynchronous frame uploads
    cudaEvent_t side_mark = nullptr;    // orders a side upload after the main stream's earlier work
    Wave wave;
    uint32_t* host_counters = nullptr;   // pinned: alive-ray counts read between rounds
    uint32_t* host_alive = nullptr;      // pinned: alive rays per request slot (serving)
    uint32_t host_alive_n = 0;
    int sms = 0;
    // launch shapes of the render wavefront (insta_tuning_set / insta_autotune); zero = built-in
    insta_tuning tune{};
    DevBuf tune_rgba, tune_depth;   // insta_autotune's device outputs
    // statistics: kernel launches issued by the library, optional per-stage CUDA-event timing
    uint64_t launches = 0;
    bool timing = false;
    std::vector<cudaEvent_t> event_pool;
    size_t events_used = 0;
    std::vector<std::pair<int, size_t>> timed;   // (stage, index of the start event)
    double stage_ms[INSTA_STAGE_COUNT] = {};
    uint32_t stage_calls[INSTA_STAGE_COUNT] = {};

    cudaEvent_t next_event() {
        if (events_used == event_pool.size()) {
            cudaEvent_t e;
            CK(cudaEventCreate(&e));
            event_pool.push_back(e);
        }
        return event_pool[events_used++];
    }
    void collect_timings() {
        if (timed.empty()) return;
        CK(cudaStreamSynchronize(stream));
        for (auto& t : timed) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, event_pool[t.second], event_pool[t.second + 1]));
            stage_ms[t.first] += ms;
            stage_calls[t.first] += 1;
        }
        timed.clear();
        events_used = 0;
    }

    void* alloc(DevBuf& b, size_t bytes) {
        if (b.p && b.bytes >= bytes) return b.p;
        release(b);
        if (budget && used + bytes > budget)
            fail(INSTA_ERR_BUDGET, "device budget exceeded: %llu + %zu > %llu bytes", (unsigned long long)used, bytes,
                 (unsigned long long)budget);
        CK(cudaMalloc(&b.p, bytes));
        b.bytes = bytes;
        used += bytes;
        return b.p;
    }
    void release(DevBuf& b) {
        if (b.p) {
            cudaFree(b.p);
            used -= b.bytes;
        }
        b.p = nullptr;
        b.bytes = 0;
    }
    // Read and clear the device error word (synchronises the stream).
    void check_device() {
        CK(cudaStreamSynchronize(stream));
        if (copy) CK(cudaStreamSynchronize(copy));
        uint32_t e = 0;
        CK(cudaMemcpy(&e, err_dev, sizeof(e), cudaMemcpyDeviceToHost));
        if (e) {
            CK(cudaMemset(err_dev, 0, sizeof(uint32_t)));
            fail(INSTA_ERR_DEVICE, "device error word 0x%x (%s%s%s%s)", e, (e & INSTA_DEVERR_STACK) ? "stack overflow " : "",
                 (e & INSTA_DEVERR_TIMEOUT) ? "wait timeout " : "", (e & INSTA_DEVERR_NO_TRI) ? "no triangle " : "",
                 (e & INSTA_DEVERR_MARCH) ? "march guard" : "");
        }
    }
    Avatar& avatar(int id, bool create = false) {
        auto it = avatars.find(id);
        if (it == avatars.end()) {
            if (!create) fail(INSTA_ERR_NOT_READY, "avatar %d has no canonical mesh", id);
            it = avatars.emplace(id, std::make_unique<Avatar>()).first;
        }
        return *it->second;
    }
};

namespace {

// Brackets the launches of one stage: counts its kernels and, with timing on, records a CUDA
// event pair on the context's stream around them.
struct Stage {
    insta_ctx* ctx;
    int stage;
    Stage(insta_ctx* c, int st, int kernels) : ctx(c), stage(st) {
        ctx->launches += (uint64_t)kernels;
        if (ctx->timing) {
            if (ctx->events_used + 2 > 4096) ctx->collect_timings();
            ctx->timed.push_back({stage, ctx->events_used});
            CK(cudaEventRecord(ctx->next_event(), ctx->stream));
        }
    }
    ~Stage() {
        if (ctx->timing) {
            if (ctx->events_used < ctx->event_pool.size() || ctx->event_pool.size() < 8192) {
                cudaEvent_t e = nullptr;
                try { e = ctx->next_event(); } catch (...) { return; }
                cudaEventRecord(e, ctx->stream);
            }
        }
    }
};

template <typename F>
int guarded(insta_ctx* ctx, F&& f) {
    if (!ctx) return INSTA_ERR_INVALID_ARG;
    try {
        int dev = -1;
        cudaGetDevice(&dev);
        if (dev != ctx->device) CK(cudaSetDevice(ctx->device));
        f();
        return INSTA_OK;
    } catch (const Failure& e) {
        ctx->last_error = e.what();
        return e.code;
    } catch (const std::exception& e) {
        ctx->last_error = e.what();
        return INSTA_ERR_CUDA;
    }
}

// TinyMesh::get_triangle_3_neighbours (src/tiny_mesh.cu:316-371): faces sharing an edge,
// sorted by id, self removed, padded with -1 (extra entries past 3 are dropped).
std::vector<int32_t> triangle_neighbours(const std::vector<int32_t>& faces, int F, int V) {
    std::vector<std::vector<int32_t>> vf(V);
    for (int f = 0; f < F; ++f)
        for (int k = 0; k < 3; ++k) vf[faces[f * 3 + k]].push_back(f);
    std::vector<int32_t> adj((size_t)F * 3, -1);
    for (int f = 0; f < F; ++f) {
        std::set<int32_t> ids;
        const int e[3][2] = {{0, 1}, {0, 2}, {1, 2}};
        for (auto& ed : e) {
            const auto& A = vf[faces[f * 3 + ed[0]]];
            const auto& B = vf[faces[f * 3 + ed[1]]];
            for (int32_t x : A)
                if (std::find(B.begin(), B.end(), x) != B.end()) ids.insert(x);
        }
        int k = 0;
        for (int32_t id : ids)
            if (id != f && k < 3) adj[(size_t)f * 3 + k++] = id;
    }
    return adj;
}

void host_copy(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s));
}

bool is_device_ptr(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

float level_scale_host(float b, uint32_t base, uint32_t l) { return exp2f((float)l * log2f(b)) * (float)base - 1.0f; }

struct FieldLayout {
    uint64_t layer_off[8];
    uint32_t layer_n[8], layer_k[8];
    int n_density, n_rgb;
    uint64_t table_off, total;
    uint32_t lvl_res[INSTA_MAX_HASH_LEVELS], lvl_size[INSTA_MAX_HASH_LEVELS];
    uint64_t lvl_off[INSTA_MAX_HASH_LEVELS];
    float lvl_scale[INSTA_MAX_HASH_LEVELS];
    float b;
};

FieldLayout field_layout(const insta_field_desc& d) {
    if (d.n_levels == 0 || d.n_levels > INSTA_MAX_HASH_LEVELS) fail(INSTA_ERR_UNSUPPORTED, "n_levels must be 1..%d", INSTA_MAX_HASH_LEVELS);
    const uint32_t F = d.n_features_per_level;
    if (F != 2 && F != 4 && F != 8) fail(INSTA_ERR_UNSUPPORTED, "n_features_per_level must be 2, 4 or 8");
    // the encode writes 8-feature groups (four levels of two, two of four, one of eight)
    if ((d.n_levels * F) % 8 != 0 || d.n_levels * F < 16 || d.n_levels * F > 128)
        fail(INSTA_ERR_UNSUPPORTED, "n_levels x n_features_per_level must be a multiple of 8 in 16..128");
    if (d.n_extra_dims != 0 && d.n_extra_dims != 16) fail(INSTA_ERR_UNSUPPORTED, "n_extra_dims must be 0 or 16");
    if (d.density_neurons != 64 || d.rgb_neurons != 64) fail(INSTA_ERR_UNSUPPORTED, "MLP width must be 64");
    if (d.density_output_dims != 16) fail(INSTA_ERR_UNSUPPORTED, "density_output_dims must be 16");
    if (d.density_hidden_layers < 1 || d.density_hidden_layers > 3 || d.rgb_hidden_layers < 1 || d.rgb_hidden_layers > 4)
        fail(INSTA_ERR_UNSUPPORTED, "hidden layer counts out of range");
    if (d.log2_hashmap_size < 8 || d.log2_hashmap_size > 24) fail(INSTA_ERR_UNSUPPORTED, "log2_hashmap_size out of range");
    if (d.precision > 2) fail(INSTA_ERR_UNSUPPORTED, "precision must be FP16, BF16 or FP8");
    FieldLayout L{};
    float b = d.per_level_scale;
    if (!(b > 0.f)) b = expf(logf(2048.0f * (float)d.aabb_scale / (float)d.base_resolution) / (float)(d.n_levels - 1));
    L.b = b;
    uint64_t off = 0;
    int li = 0;
    uint32_t n_in = d.n_levels * F + d.n_extra_dims;
    std::vector<uint32_t> w = {n_in};
    for (uint32_t h = 0; h < d.density_hidden_layers; ++h) w.push_back(64);
    w.push_back(16);
    for (size_t k = 0; k + 1 < w.size(); ++k) { L.layer_off[li] = off; L.layer_n[li] = w[k + 1]; L.layer_k[li] = w[k]; off += (uint64_t)w[k + 1] * w[k]; ++li; }
    L.n_density = li;
    w = {32};
    for (uint32_t h = 0; h < d.rgb_hidden_layers; ++h) w.push_back(64);
    w.push_back(16);
    for (size_t k = 0; k + 1 < w.size(); ++k) { L.layer_off[li] = off; L.layer_n[li] = w[k + 1]; L.layer_k[li] = w[k]; off += (uint64_t)w[k + 1] * w[k]; ++li; }
    L.n_rgb = li - L.n_density;
    L.table_off = off;
    uint64_t T = 1ull << d.log2_hashmap_size, eoff = 0;
    for (uint32_t l = 0; l < d.n_levels; ++l) {
        float s = level_scale_host(b, d.base_resolution, l);
        uint32_t res = (uint32_t)ceilf(s) + 1u;
        uint64_t r3 = (uint64_t)res * res * res;
        uint64_t sz = std::min((r3 + 7) / 8 * 8, T);
        L.lvl_res[l] = res; L.lvl_size[l] = (uint32_t)sz; L.lvl_off[l] = eoff; L.lvl_scale[l] = s;
        eoff += sz;
    }
    L.total = off + eoff * F;
    return L;
}

float half_to_float(uint16_t h) {
    uint32_t sign = (h >> 15) & 1u, exp = (h >> 10) & 0x1fu, man = h & 0x3ffu;
    float f;
    if (exp == 0) f = std::ldexp((float)man, -24);
    else if (exp == 31) f = man ? NAN : INFINITY;
    else f = std::ldexp((float)(man | 0x400u), (int)exp - 25);
    return sign ? -f : f;
}

// FP8 E4M3 encoding of x: nearest representable value, ties to even, saturating at +-448 (the
// SATFINITE conversion of the device); NaN -> 0x7f.
uint8_t float_to_e4m3(float x) {
    if (x != x) return 0x7f;
    const uint8_t sign = std::signbit(x) ? 0x80 : 0x00;
    const float a = std::fabs(x);
    if (a >= 448.0f) return sign | 0x7e;
    if (a < 0.015625f) {                          // subnormals: multiples of 2^-9
        const float m = std::nearbyint(a * 512.0f);   // 0..8; 8 is the smallest normal
        if (m >= 8.0f) return sign | 0x08;
        return sign | (uint8_t)m;
    }
    int e;
    std::frexp(a, &e);                            // a = m 2^e, m in [0.5, 1)
    float q = std::nearbyint(std::ldexp(a, 4 - e));   // 8..16: the leading bit and 3 mantissa bits
    if (q >= 16.0f) { q = 8.0f; ++e; }
    const int E = e - 1 + 7;                      // biased exponent
    if (E > 15 || (E == 15 && q > 14.0f)) return sign | 0x7e;
    return sign | (uint8_t)(E << 3) | (uint8_t)((int)q - 8);
}

uint16_t half_to_bf16_bits(uint16_t h) {
    // exact FP16 -> FP32, then round-to-nearest-even to BF16
    uint32_t sign = (h >> 15) & 1u, exp = (h >> 10) & 0x1fu, man = h & 0x3ffu;
    float f;
    if (exp == 0) f = std::ldexp((float)man, -24);
    else if (exp == 31) f = man ? NAN : INFINITY;
    else f = std::ldexp((float)(man | 0x400u), (int)exp - 25);
    if (sign) f = -f;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

Frame& get_frame(Avatar& a, int frame) {
    auto it = a.frames.find(frame);
    if (it == a.frames.end()) fail(INSTA_ERR_NOT_READY, "frame %d was not uploaded", frame);
    return it->second;
}

// Make the context's stream wait for an asynchronous upload of the frame, if one is pending.
void wait_frame(insta_ctx* ctx, Frame& f) {
    if (!f.pending) return;
    CK(cudaStreamWaitEvent(ctx->stream, f.ready, 0));
    f.pending = false;
}

// The frame, with the context's stream ordered after its pending asynchronous upload.
Frame& use_frame(insta_ctx* ctx, Avatar& a, int frame) {
    Frame& f = get_frame(a, frame);
    wait_frame(ctx, f);
    return f;
}

// Every frame of the avatar (work that picks frames per record).
void wait_all_frames(insta_ctx* ctx, Avatar& a) {
    for (auto& kv : a.frames) wait_frame(ctx, kv.second);
}

DeformView deform_view(const Avatar& a) {
    DeformView dv{};
    dv.canon = static_cast<const TriFrame*>(a.canon_frames.p);
    dv.adjacency = static_cast<const int32_t*>(a.adjacency.p);
    dv.disable_interp = (a.flags & INSTA_FLAG_DISABLE_INTERP) ? 1 : 0;
    for (int k = 0; k < 3; ++k) { dv.aabb_min[k] = a.train_min[k]; dv.aabb_max[k] = a.train_max[k]; }
    return dv;
}

RenderView render_view(const Avatar& a, const insta_render_desc& r) {
    RenderView rv{};
    rv.width = r.width; rv.height = r.height;
    rv.focal[0] = r.focal_length[0]; rv.focal[1] = r.focal_length[1];
    rv.screen_center[0] = r.screen_center[0]; rv.screen_center[1] = r.screen_center[1];
    std::memcpy(rv.cam, r.camera, sizeof(rv.cam));
    for (int k = 0; k < 3; ++k) {
        rv.aabb_min[k] = a.render_min[k]; rv.aabb_max[k] = a.render_max[k];
        rv.train_min[k] = a.train_min[k]; rv.train_max[k] = a.train_max[k];
    }
    rv.cone_angle = r.cone_angle;
    rv.min_transmittance = r.min_transmittance;
    rv.spp = r.spp;
    rv.max_samples_per_ray = r.max_samples_per_ray ? r.max_samples_per_ray : 1024u;
    rv.snap_to_pixel_centers = r.snap_to_pixel_centers ? 1 : 0;
    rv.frame_id = r.frame;
    rv.linear_colors = r.linear_colors ? 1 : 0;
    return rv;
}

void check_request(const insta_render_desc* r) {
    if (!r) fail(INSTA_ERR_INVALID_ARG, "null request");
    if (r->width <= 0 || r->height <= 0 || (int64_t)r->width * r->height > (int64_t)1 << 25)
        fail(INSTA_ERR_INVALID_ARG, "bad resolution %dx%d", r->width, r->height);
    if (!(r->focal_length[0] > 0.f) || !(r->focal_length[1] > 0.f)) fail(INSTA_ERR_INVALID_ARG, "focal length must be positive");
    if (r->cone_angle < 0.f) fail(INSTA_ERR_INVALID_ARG, "cone_angle must be >= 0");
    if (r->out_samples && !is_device_ptr(r->out_samples)) fail(INSTA_ERR_INVALID_ARG, "out_samples must be device memory");
}

// Largest number of samples one round may produce (bounds the per-sample scratch, ~160 B each),
// and the most pixels (ray slots) one batch may hold.
constexpr uint64_t kMaxRoundSamples = 32ull << 20;
constexpr uint64_t kMaxBatchPixels = 1ull << 25;
// Samples per alive ray per round: at most kMaxSteps, built-in kDefaultSteps.  With 64 a 512x512
// frame of the benchmark takes nearly all of its samples in the first round (with 32, a second
// round of about a tenth of them ran at low occupancy: 1.89 -> 1.76 ms per frame); the round
// budget caps it for large batches.
constexpr uint32_t kMaxSteps = 128, kDefaultSteps = 64;
static_assert(kMaxSteps <= (1u << (32 - kStepShift)), "step index must fit beside the ray slot");

// The wavefront's launch shapes under the context's tuning (zero fields: built-in choices).
uint32_t tune_steps(const insta_ctx* ctx) { return ctx->tune.max_steps_per_round ? ctx->tune.max_steps_per_round : kDefaultSteps; }
// Built-in sort grid: 64^3 cells per request while the bins stay within 4 Mi (a round's
// counting sort clears and scans them), else 32^3 (16^3 beyond 128 request slots).
uint32_t tune_cell_bits(const insta_ctx* ctx, uint32_t slots) {
    if (ctx->tune.sort_cell_bits) return ctx->tune.sort_cell_bits;
    uint32_t b = 18u;
    while (b > 12u && ((uint64_t)slots << b) > (4ull << 20)) b -= 3u;
    return b;
}
static_assert(kMaxBatchPixels <= (uint64_t)kRayMask + 1u, "ray slots (at most 2^25 pixels per batch) must fit below the step index");

bool same_field_layout(const Field& a, const Field& b) {
    return std::memcmp(&a.plan, &b.plan, sizeof(TilePlan)) == 0 && a.view.n_levels == b.view.n_levels &&
           a.view.n_features == b.view.n_features && a.view.n_extra == b.view.n_extra && a.view.precision == b.view.precision &&
           std::memcmp(a.view.level_scale, b.view.level_scale, sizeof(a.view.level_scale)) == 0 &&
           std::memcmp(a.view.level_res, b.view.level_res, sizeof(a.view.level_res)) == 0 &&
           std::memcmp(a.view.level_size, b.view.level_size, sizeof(a.view.level_size)) == 0 &&
           std::memcmp(a.view.level_off, b.view.level_off, sizeof(a.view.level_off)) == 0 &&
           std::memcmp(a.view.level_dense, b.view.level_dense, sizeof(a.view.level_dense)) == 0;
}

// A request's slot view: camera, frame, avatar state and output buffers (set by the caller).
ReqView request_view(insta_ctx* ctx, const insta_render_desc& r, Avatar& a, Frame& f) {
    ReqView v{};
    v.rv = render_view(a, r);
    v.fr = f.view;
    v.dv = deform_view(a);
    v.table = a.field.view.table;
    v.mlp = a.field.view.mlp_smem;
    v.bitfield = (const uint8_t*)f.bitfield.p;
    v.out_samples = r.out_samples;
    v.tiles_x = ((uint32_t)r.width + 7) / 8;
    v.tiles = v.tiles_x * (((uint32_t)r.height + 3) / 4);
    return v;
}

// The render wavefront over a table of request slots (NerfTracer::trace for many views at once,
// ngp/src/testbed_nerf.cu:2112-2244): rays of any slots can be started between rounds; each
// round marches all alive rays, sorts their samples by (slot, cell), runs deform + encode, the
// MLP tiles and the composite.  The host reads the alive count after each round, as trace does
// (:2164-2165).
struct WaveRun {
    insta_ctx* ctx = nullptr;
    uint32_t n_slots = 0;
    uint32_t steps_max = kDefaultSteps;   // samples per alive ray per round, at most
    uint64_t round_cap = 0, cap_samples = 0;
    WaveArgs W{};
    MlpArgs M{};
    int cur = 0;
    uint32_t n_alive = 0;
    uint32_t* counters = nullptr;

    // deform + encode + MLP as one kernel: FP16 / BF16 fields when the tuning asks for it
    // (the fused kernel's 16 KiB tile holds the hash rows and the SH rows: at most 48 + 16 columns;
    // it encodes two features per level)
    bool fused_field() const { return W.fv.precision != 2 && W.fv.n_features == 2 && W.k_in <= 48u && ctx->tune.fused_field_stage; }

    RayBuf rays(int b) {
        Wave& w = ctx->wave;
        return RayBuf{(float4*)w.rays[b][0].p, (float4*)w.rays[b][1].p, (float4*)w.rays[b][2].p, (float4*)w.rays[b][3].p};
    }

    // Scratch for up to max_rays alive rays over n_slots slots sharing `field`'s layout.
    void setup(insta_ctx* c, const Field& field, uint32_t slots, uint64_t max_rays, bool per_request_counts,
               uint64_t max_round_samples = kMaxRoundSamples) {
        ctx = c;
        n_slots = slots;
        const FieldView& fv = field.view;
        const TilePlan& P = field.plan;
        Wave& w = ctx->wave;
        steps_max = tune_steps(ctx);
        // at least one sample per alive ray fits a round: the march takes max(1, cap / alive) steps
        // per ray and writes into buffers of cap_samples (max_rays <= 2^25 = kMaxRoundSamples)
        round_cap = std::min<uint64_t>(max_rays * steps_max, std::max(max_rays, std::min(max_round_samples, kMaxRoundSamples)));
        cap_samples = (round_cap + (uint64_t)slots * 128 + 127) / 128 * 128;
        const uint32_t cell_bits = sort_cell_bits(slots, tune_cell_bits(ctx, slots));
        const uint64_t n_bins = (uint64_t)slots << cell_bits;
        if (w.cap_rays < max_rays) {
            for (int b = 0; b < 2; ++b)
                for (int k = 0; k < 4; ++k) ctx->alloc(w.rays[b][k], (size_t)max_rays * 16);
            ctx->alloc(w.n_round, (size_t)max_rays * 4);
            w.cap_rays = (uint32_t)max_rays;
        }
        ctx->alloc(w.tiles, cap_samples / 128 * P.tile_bytes);
        ctx->alloc(w.aux, cap_samples * sizeof(float2));
        ctx->alloc(w.samples, cap_samples * sizeof(float4));
        ctx->alloc(w.march_t, cap_samples * sizeof(float));
        ctx->alloc(w.sample_ray, cap_samples * sizeof(uint32_t));
        ctx->alloc(w.sample_index, cap_samples * sizeof(uint32_t));
        ctx->alloc(w.sample_key, cap_samples * sizeof(uint32_t));
        ctx->alloc(w.sample_order, cap_samples * sizeof(uint32_t));
        ctx->alloc(w.sort_bins, (n_bins + n_bins / kSortBlock) * sizeof(uint32_t));
        ctx->alloc(w.out, cap_samples * sizeof(uint2));
        if (fv.precision != 0) ctx->alloc(w.out_f32, cap_samples * sizeof(float4));
        ctx->alloc(w.counters, 64);
        ctx->alloc(w.req_table, (size_t)slots * sizeof(ReqView));
        ctx->alloc(w.req_meta, (size_t)(slots + 1) * 2 * sizeof(uint32_t) + (size_t)slots * sizeof(uint32_t));
        ctx->alloc(w.init_meta, (size_t)(2 * slots + 1) * sizeof(uint32_t));
        if (!ctx->host_counters) CK(cudaMallocHost(&ctx->host_counters, 64));
        if (!ctx->host_alive || ctx->host_alive_n < slots) {
            if (ctx->host_alive) cudaFreeHost(ctx->host_alive);
            CK(cudaMallocHost(&ctx->host_alive, (size_t)slots * sizeof(uint32_t)));
            ctx->host_alive_n = slots;
        }
        counters = (uint32_t*)w.counters.p;   // [0], [1]: ping-pong alive counts; [2]: round samples; [3]: padded
        W = WaveArgs{};
        W.reqs = (const ReqView*)w.req_table.p;
        W.n_reqs = slots;
        W.cell_bits = cell_bits;
        W.fv = fv;
        W.tiles = (uint8_t*)w.tiles.p;
        W.tile_bytes = P.tile_bytes;
        W.k_in = P.k_in;
        W.aux = (float2*)w.aux.p;
        W.samples = (float4*)w.samples.p;
        W.march_t = (float*)w.march_t.p;
        W.sample_ray = (uint32_t*)w.sample_ray.p;
        W.sample_index = (uint32_t*)w.sample_index.p;
        W.sample_key = (uint32_t*)w.sample_key.p;
        W.sample_order = (uint32_t*)w.sample_order.p;
        W.sort_bins = (uint32_t*)w.sort_bins.p;
        W.sort_block_sums = W.sort_bins + n_bins;
        W.req_start = (uint32_t*)w.req_meta.p;
        W.req_seg = W.req_start + (slots + 1);
        W.req_alive = per_request_counts ? W.req_seg + (slots + 1) : nullptr;
        W.init_tile = (const uint32_t*)w.init_meta.p;
        W.init_slot = W.init_tile + (slots + 1);
        W.n_samples_round = counters + 2;
        W.n_samples_padded = counters + 3;
        W.nearest_work = counters + 4;
        W.out = (const uint2*)w.out.p;
        W.out_f32 = (const float4*)w.out_f32.p;
        W.n_round = (uint32_t*)w.n_round.p;
        W.sample_counter = ctx->sample_counter;
        W.top_nodes = ctx->tune.bvh_top_nodes;
        if (ctx->timing && !ctx->walk_stats) {
            CK(cudaMalloc(&ctx->walk_stats, 8 * sizeof(unsigned long long)));
            CK(cudaMemset(ctx->walk_stats, 0, 8 * sizeof(unsigned long long)));
        }
        W.walk_stats = ctx->timing ? ctx->walk_stats : nullptr;
        W.err = ctx->err_dev;
        M = MlpArgs{};
        M.fv = fv; M.plan = P; M.tiles = W.tiles;
        M.out = (uint2*)w.out.p; M.out_f32 = (float4*)w.out_f32.p; M.err = ctx->err_dev;
        M.n_alive = W.n_samples_padded;
        M.seg = W.req_seg; M.reqs = W.reqs; M.n_reqs = slots;
        cur = 0;
        n_alive = 0;
        CK(cudaMemsetAsync(ctx->sample_counter, 0, sizeof(unsigned long long), ctx->stream));
        CK(cudaMemsetAsync(counters, 0, 24, ctx->stream));   // alive counts, round counts, nearest-stage work
        if (W.req_alive) CK(cudaMemsetAsync(W.req_alive, 0, (size_t)slots * sizeof(uint32_t), ctx->stream));
    }

    void upload_table(const ReqView* views) {
        CK(cudaMemcpyAsync(ctx->wave.req_table.p, views, (size_t)n_slots * sizeof(ReqView), cudaMemcpyHostToDevice, ctx->stream));
    }

    // Start the rays of the given slots, appended to the current alive list.  `tiles[k]` is slot
    // slots[k]'s tile count.  Without read_back, the new pixels bound the alive count (no host
    // round trip).
    void start(const uint32_t* slots, const uint32_t* tiles, uint32_t n, bool read_back) {
        std::vector<uint32_t> meta((size_t)2 * n + 1);
        uint32_t total = 0;
        for (uint32_t k = 0; k < n; ++k) { meta[k] = total; total += tiles[k]; meta[n + 1 + k] = slots[k]; }
        meta[n] = total;
        // init_tile then init_slot, packed for this launch
        CK(cudaMemcpyAsync(ctx->wave.init_meta.p, meta.data(), meta.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
        W.init_tile = (const uint32_t*)ctx->wave.init_meta.p;
        W.init_slot = W.init_tile + (n + 1);
        W.n_init = n;
        W.rays_out = rays(cur);
        W.n_alive_out = counters + cur;
        { Stage st(ctx, INSTA_STAGE_RAY_INIT, 1); CK(launch_ray_init(W, total, ctx->stream)); }
        if (read_back) n_alive = read_alive();
        else n_alive += total * 32u;   // upper bound: every pixel alive
    }

    uint32_t read_alive() {
        CK(cudaMemcpyAsync(ctx->host_counters, counters + cur, 4, cudaMemcpyDeviceToHost, ctx->stream));
        if (W.req_alive)
            CK(cudaMemcpyAsync(ctx->host_alive, W.req_alive, (size_t)n_slots * 4, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        return ctx->host_counters[0];
    }

    // All remaining rounds on the device: one launch of a CUDA graph whose conditional while node
    // runs pairs of rounds (ping-pong ray buffers) until no ray is alive or max_rounds have run.
    // The host does not wait; n_alive is not read back.
    void device_rounds(uint32_t max_rounds) {
        if (!ctx->loop_state) {
            CK(cudaMalloc(&ctx->loop_state, 64));
            CK(cudaMemset(ctx->loop_state, 0, 64));
            ctx->loop_rounds_total = reinterpret_cast<unsigned long long*>(ctx->loop_state + 8);
        }
        WaveArgs A = W, B = W;
        A.steps_dev = B.steps_dev = ctx->loop_state;
        A.rays_in = rays(cur); A.rays_out = rays(cur ^ 1);
        A.n_alive_in = counters + cur; A.n_alive_out = counters + (cur ^ 1);
        B.rays_in = rays(cur ^ 1); B.rays_out = rays(cur);
        B.n_alive_in = counters + (cur ^ 1); B.n_alive_out = counters + cur;
        A.n_init = B.n_init = 0; A.init_tile = B.init_tile = nullptr; A.init_slot = B.init_slot = nullptr;
        A.steps = B.steps = 0;
        std::vector<unsigned char> key(sizeof(WaveArgs) * 2 + sizeof(MlpArgs) + 16 + sizeof(insta_tuning));
        std::memcpy(key.data(), &A, sizeof(WaveArgs));
        std::memcpy(key.data() + sizeof(WaveArgs), &B, sizeof(WaveArgs));
        std::memcpy(key.data() + 2 * sizeof(WaveArgs), &M, sizeof(MlpArgs));
        std::memcpy(key.data() + 2 * sizeof(WaveArgs) + sizeof(MlpArgs), &round_cap, 8);
        std::memcpy(key.data() + 2 * sizeof(WaveArgs) + sizeof(MlpArgs) + 8, &max_rounds, 4);
        const uint32_t grid_tiles = (uint32_t)(cap_samples / 128);
        std::memcpy(key.data() + 2 * sizeof(WaveArgs) + sizeof(MlpArgs) + 12, &grid_tiles, 4);
        std::memcpy(key.data() + 2 * sizeof(WaveArgs) + sizeof(MlpArgs) + 16, &ctx->tune, sizeof(insta_tuning));
        if (!ctx->loop_exec || key != ctx->loop_key) {
            if (ctx->loop_exec) { cudaGraphExecDestroy(ctx->loop_exec); ctx->loop_exec = nullptr; }
            if (ctx->loop_graph) { cudaGraphDestroy(ctx->loop_graph); ctx->loop_graph = nullptr; }
            cudaGraph_t g;
            CK(cudaGraphCreate(&g, 0));
            ctx->loop_graph = g;
            cudaGraphConditionalHandle cond;
            CK(cudaGraphConditionalHandleCreate(&cond, g, 1u, cudaGraphCondAssignDefault));
            cudaGraphNodeParams cp{};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = cond;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t node;
            CK(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp));
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            if (!ctx->capture) CK(cudaStreamCreateWithFlags(&ctx->capture, cudaStreamNonBlocking));
            // one round's kernels on stream st
            auto round_kernels = [&](const WaveArgs& R, cudaStream_t st) -> cudaError_t {
                cudaError_t e = launch_round_begin(R.n_alive_in, R.n_alive_out, R.n_samples_round, ctx->loop_state, round_cap, steps_max, st);
                if (e == cudaSuccess) e = launch_march(R, st);
                if (e == cudaSuccess) e = launch_sort_samples(R, st);
                if (fused_field()) {
                    if (e == cudaSuccess) e = launch_nearest_stage(R, ctx->tune.deform_blocks_per_sm, st);
                    if (e == cudaSuccess) e = launch_field_fused(R, M, grid_tiles, st, ctx->tune.mlp_ctas_per_sm);
                } else {
                    if (e == cudaSuccess) e = launch_deform_encode(R, ctx->tune.deform_blocks_per_sm, st);
                    if (e == cudaSuccess) e = launch_mlp(M, grid_tiles, st, ctx->tune.mlp_ctas_per_sm, ctx->tune.mlp_slots);
                }
                if (e == cudaSuccess) e = launch_composite(R, st);
                return e;
            };
            // The body by capture: round A; round B under a conditional IF node that
            // round_mid_kernel sets only when rays are still alive (a frame whose rays all finish
            // in round A launches none of B's kernels); then the loop condition.
            CK(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
            cudaGraphConditionalHandle if_cond{};
            cudaError_t e = cudaGraphConditionalHandleCreate(&if_cond, body, 0u, 0u);
            if (e == cudaSuccess) e = round_kernels(A, ctx->stream);
            if (e == cudaSuccess) e = launch_round_mid(A.n_alive_out, B.n_alive_out, ctx->loop_state + 2, if_cond, ctx->stream);
            cudaGraph_t if_body = nullptr;
            if (e == cudaSuccess) {
                cudaStreamCaptureStatus status;
                cudaGraph_t capturing = nullptr;
                const cudaGraphNode_t* deps = nullptr;
                size_t n_deps = 0;
                e = cudaStreamGetCaptureInfo(ctx->stream, &status, nullptr, &capturing, &deps, nullptr, &n_deps);
                if (e == cudaSuccess) {
                    cudaGraphNodeParams ip{};
                    ip.type = cudaGraphNodeTypeConditional;
                    ip.conditional.handle = if_cond;
                    ip.conditional.type = cudaGraphCondTypeIf;
                    ip.conditional.size = 1;
                    cudaGraphNode_t if_node = nullptr;
                    e = cudaGraphAddNode(&if_node, capturing, deps, nullptr, n_deps, &ip);
                    if (e == cudaSuccess) {
                        if_body = ip.conditional.phGraph_out[0];
                        e = cudaStreamUpdateCaptureDependencies(ctx->stream, &if_node, nullptr, 1, cudaStreamSetCaptureDependencies);
                    }
                }
            }
            if (e == cudaSuccess) {
                e = cudaStreamBeginCaptureToGraph(ctx->capture, if_body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
                if (e == cudaSuccess) {
                    const cudaError_t eb = round_kernels(B, ctx->capture);
                    cudaGraph_t captured_b = nullptr;
                    const cudaError_t ee = cudaStreamEndCapture(ctx->capture, &captured_b);
                    e = eb != cudaSuccess ? eb : ee;
                }
            }
            if (e == cudaSuccess)
                e = launch_round_end(B.n_alive_out, ctx->loop_state + 1, ctx->loop_state + 2, ctx->loop_rounds_total, max_rounds, cond, ctx->stream);
            cudaGraph_t captured = nullptr;
            const cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &captured);
            CK(e);
            CK(e2);
            CK(cudaGraphInstantiate(&ctx->loop_exec, g, 0));
            ctx->loop_key = key;
        }
        ctx->loop_round_kernels = fused_field() ? 9u : 10u;
        CK(cudaMemsetAsync(ctx->loop_state + 1, 0, 4, ctx->stream));
        CK(cudaGraphLaunch(ctx->loop_exec, ctx->stream));   // its kernels are counted from the device's round total
    }

    // One round over all alive rays; afterwards n_alive (and host_alive per slot) are current.
    // Without read_back the host does not wait: n_alive stays an upper bound (rays only finish),
    // and the next round's kernels take the count from the device.
    void round(bool read_back = true) {
        const uint32_t steps = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(steps_max, round_cap / std::max(1u, n_alive)));
        W.steps = steps;
        W.rays_in = rays(cur);
        W.rays_out = rays(cur ^ 1);
        W.n_alive_in = counters + cur;
        W.n_alive_out = counters + (cur ^ 1);
        CK(cudaMemsetAsync(counters + (cur ^ 1), 0, 4, ctx->stream));
        CK(cudaMemsetAsync(counters + 2, 0, 4, ctx->stream));
        { Stage st(ctx, INSTA_STAGE_MARCH, 1); CK(launch_march(W, ctx->stream)); }
        { Stage st(ctx, INSTA_STAGE_SORT, 4); CK(launch_sort_samples(W, ctx->stream)); }
        { Stage st(ctx, INSTA_STAGE_NEAREST, 1); CK(launch_nearest_stage(W, ctx->tune.deform_blocks_per_sm, ctx->stream)); }
        if (fused_field()) {
            // the fused deform + encode + MLP kernel under the MLP stage
            Stage st(ctx, INSTA_STAGE_MLP, 1);
            CK(launch_field_fused(W, M, (uint32_t)(cap_samples / 128), ctx->stream, ctx->tune.mlp_ctas_per_sm));
        } else {
            { Stage st(ctx, INSTA_STAGE_DEFORM_ENCODE, 1); CK(launch_map_encode(W, ctx->tune.deform_blocks_per_sm, ctx->stream)); }
            { Stage st(ctx, INSTA_STAGE_MLP, 1); CK(launch_mlp(M, (uint32_t)(cap_samples / 128), ctx->stream, ctx->tune.mlp_ctas_per_sm, ctx->tune.mlp_slots)); }
        }
        { Stage st(ctx, INSTA_STAGE_COMPOSITE, 1); CK(launch_composite(W, ctx->stream)); }
        cur ^= 1;
        if (read_back) n_alive = read_alive();
    }
};

// The context's copy stream for device -> host output copies and the events of the
// double-buffered insta_render_async staging, created together on first use.
void ensure_copy_stream(insta_ctx* ctx) {
    if (ctx->copy) return;
    CK(cudaStreamCreateWithFlags(&ctx->copy, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) CK(cudaEventCreateWithFlags(&ctx->async_free[k], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ctx->async_done, cudaEventDisableTiming));
}

// Testbed::render_nerf for a batch of requests (avatars, frames, cameras, resolutions) through one
// wavefront; the request slots are the batch.
void render_batch(insta_ctx* ctx, const insta_render_desc* reqs, int n, float* const* out_rgba, float* const* out_depth,
                  bool async_host = false) {
    if (n <= 0 || (uint32_t)n > kMaxRequests) fail(INSTA_ERR_INVALID_ARG, "batch size %d outside 1..%u", n, kMaxRequests);
    std::vector<ReqView> views((size_t)n);
    const Field* field0 = nullptr;
    uint64_t total_pix = 0, host_pix = 0;
    uint32_t max_spr = 0;
    std::vector<int> on_host((size_t)n, 0);
    std::vector<uint32_t> slots((size_t)n), tiles((size_t)n);
    for (int i = 0; i < n; ++i) {
        const insta_render_desc* r = reqs + i;
        check_request(r);
        if (!out_rgba[i] || !out_depth[i]) fail(INSTA_ERR_INVALID_ARG, "null output buffers for request %d", i);
        Avatar& a = ctx->avatar(r->avatar);
        if (!a.field.ready) fail(INSTA_ERR_NOT_READY, "avatar %d has no field parameters", r->avatar);
        Frame& f = use_frame(ctx, a, r->frame);
        if (!f.has_occupancy) fail(INSTA_ERR_NOT_READY, "frame %d has no occupancy bitfield", r->frame);
        if (!field0) field0 = &a.field;
        else if (!same_field_layout(*field0, a.field))
            fail(INSTA_ERR_UNSUPPORTED, "requests of one batch must share the field layout (request %d differs)", i);
        views[(size_t)i] = request_view(ctx, *r, a, f);
        slots[(size_t)i] = (uint32_t)i;
        tiles[(size_t)i] = views[(size_t)i].tiles;
        const uint64_t px = (uint64_t)r->width * r->height;
        total_pix += px;
        on_host[(size_t)i] = !(is_device_ptr(out_rgba[i]) && is_device_ptr(out_depth[i]));
        if (on_host[(size_t)i]) host_pix += px;
        max_spr = std::max(max_spr, views[(size_t)i].rv.max_samples_per_ray);
    }
    // a round takes at least one sample per alive ray: the pixels must fit one round's buffers
    if (total_pix > kMaxBatchPixels) fail(INSTA_ERR_INVALID_ARG, "a batch holds at most 2^25 pixels, got %llu", (unsigned long long)total_pix);
    // outputs: device pointers directly, host pointers through one staging buffer
    float* stage_rgba = nullptr;
    float* stage_depth = nullptr;
    int async_k = -1;
    if (host_pix && async_host) {
        // the staging pair the copy stream released last; the render waits for its copy to end
        async_k = ctx->async_next;
        ensure_copy_stream(ctx);
        if (ctx->async_used[async_k]) CK(cudaStreamWaitEvent(ctx->stream, ctx->async_free[async_k], 0));
        stage_rgba = (float*)ctx->alloc(ctx->async_rgba[async_k], host_pix * 16);
        stage_depth = (float*)ctx->alloc(ctx->async_depth[async_k], host_pix * 4);
    } else if (host_pix) {
        stage_rgba = (float*)ctx->alloc(ctx->out_rgba, host_pix * 16);
        stage_depth = (float*)ctx->alloc(ctx->out_depth, host_pix * 4);
    }
    // per-request expression dims (host arrays) into one device block
    const uint32_t n_extra = field0->view.n_extra;
    std::vector<float> extra;
    if (n_extra) {
        extra.assign((size_t)n * n_extra, 0.f);
        for (int i = 0; i < n; ++i)
            if (reqs[i].extra_dims) std::memcpy(extra.data() + (size_t)i * n_extra, reqs[i].extra_dims, n_extra * 4);
        ctx->alloc(ctx->extra, extra.size() * 4);
    }
    {
        uint64_t off = 0;
        for (int i = 0; i < n; ++i) {
            ReqView& v = views[(size_t)i];
            if (on_host[(size_t)i]) {
                v.out_rgba = stage_rgba + off * 4;
                v.out_depth = stage_depth + off;
                off += (uint64_t)reqs[i].width * reqs[i].height;
            } else {
                v.out_rgba = out_rgba[i];
                v.out_depth = out_depth[i];
            }
            v.extra = n_extra ? (const float*)ctx->extra.p + (size_t)i * n_extra : nullptr;
        }
    }
    WaveRun run;
    run.setup(ctx, *field0, (uint32_t)n, total_pix, false);
    {
        // one weight image for every request (one avatar, or avatars sharing one): the MLP stage
        // can keep it resident once per SM
        bool same = true;
        for (int i = 1; i < n; ++i) same = same && views[(size_t)i].mlp == views[0].mlp;
        run.M.single = same ? views[0].mlp : nullptr;
        run.M.batch = n > 1 ? 1u : 0u;
    }
    if (n_extra) CK(cudaMemcpyAsync(ctx->extra.p, extra.data(), extra.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    run.upload_table(views.data());
    // the first round's step count needs the alive count only when all pixels could not take
    // steps_max samples each; otherwise the pixel count stands in for it (no host round trip)
    run.start(slots.data(), tiles.data(), (uint32_t)n, total_pix * run.steps_max > run.round_cap);
    // while every ray can take steps_max samples per round, the first round is issued without a
    // host read of its alive count (most frames finish in two rounds: one host wait, not two)
    uint32_t round = 0;
    if (!ctx->timing && run.n_alive > 0) {
        // the whole loop on the device (one CUDA-graph launch); per-stage timing needs the
        // host-driven rounds below, which run the same kernels
        run.device_rounds(max_spr + 2);
    } else {
        if (total_pix * run.steps_max <= run.round_cap && run.n_alive > 0) {
            run.round(false);
            ++round;
        }
        for (; run.n_alive > 0 && round < max_spr + 2; ++round) run.round();
    }
    if (host_pix) {
        cudaStream_t cs = ctx->stream;
        if (async_k >= 0) {
            CK(cudaEventRecord(ctx->async_done, ctx->stream));
            CK(cudaStreamWaitEvent(ctx->copy, ctx->async_done, 0));
            cs = ctx->copy;
        }
        uint64_t off = 0;
        for (int i = 0; i < n; ++i) {
            if (!on_host[(size_t)i]) continue;
            const size_t px = (size_t)reqs[i].width * reqs[i].height;
            CK(cudaMemcpyAsync(out_rgba[i], stage_rgba + off * 4, px * 16, cudaMemcpyDeviceToHost, cs));
            CK(cudaMemcpyAsync(out_depth[i], stage_depth + off, px * 4, cudaMemcpyDeviceToHost, cs));
            off += px;
        }
        if (async_k >= 0) {
            CK(cudaEventRecord(ctx->async_free[async_k], ctx->copy));
            ctx->async_used[async_k] = true;
            ctx->async_next = async_k ^ 1;
        } else {
            ctx->check_device();
        }
    }
}

// Device buffers and view of one uploaded frame; copies its vertices in.
Frame& prepare_frame(insta_ctx* ctx, Avatar& a, int frame, const float* verts, cudaStream_t stream = nullptr) {
    Frame& f = a.frames[frame];
    if (!stream || stream == ctx->stream) wait_frame(ctx, f);   // an async upload of it still in flight
    // an LBVH with leaves of <= 2 triangles has at most F - 1 internal nodes
    const int max_nodes = std::max(1, a.F);
    ctx->alloc(f.verts, (size_t)a.V * 12);
    ctx->alloc(f.frames, (size_t)a.F * sizeof(TriFrame));
    ctx->alloc(f.leaf_tris, (size_t)a.F * (INSTA_TRI_F4 + 2) * 16);   // records, then the bounding disks
    ctx->alloc(f.nodes, (size_t)max_nodes * 112);
    host_copy(f.verts.p, verts, (size_t)a.V * 12, stream ? stream : ctx->stream);
    f.view.leaf_tris = static_cast<const float4*>(f.leaf_tris.p);
    f.view.leaf_bounds = f.view.leaf_tris + (size_t)a.F * INSTA_TRI_F4;
    f.view.nodes = static_cast<const float4*>(f.nodes.p);
    f.view.frames = static_cast<const TriFrame*>(f.frames.p);
    f.view.n_tris = a.F;
    f.view.n_nodes = max_nodes;
    f.has_occupancy = false;
    a.table_dirty = true;
    return f;
}

// Device table of the avatar's frame views, indexed by frame id (the `holder` lookup of warp).
void refresh_frame_table(insta_ctx* ctx, Avatar& a) {
    if (!a.table_dirty) return;
    int max_id = a.frames.empty() ? -1 : a.frames.rbegin()->first;
    std::vector<FrameView> table((size_t)std::max(1, max_id + 1));
    for (auto& fv : table) std::memset(&fv, 0, sizeof(fv));
    for (auto& kv : a.frames) table[kv.first] = kv.second.view;
    ctx->alloc(a.frame_table, table.size() * sizeof(FrameView));
    CK(cudaMemcpyAsync(a.frame_table.p, table.data(), table.size() * sizeof(FrameView), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    a.table_frames = (uint32_t)(max_id + 1);
    a.table_dirty = false;
}

}  // namespace

extern "C" {

int insta_ctx_create(int device, void* cuda_stream, uint64_t budget_bytes, insta_ctx** out) {
    if (!out) return INSTA_ERR_INVALID_ARG;
    *out = nullptr;
    auto ctx = std::make_unique<insta_ctx>();
    ctx->device = device;
    ctx->budget = budget_bytes;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return INSTA_ERR_CUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess) return INSTA_ERR_CUDA;
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
    if (major != 10) return INSTA_ERR_UNSUPPORTED;   // tcgen05 kernels are built for sm_103a only
    cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
    if (cuda_stream) ctx->stream = static_cast<cudaStream_t>(cuda_stream);
    else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return INSTA_ERR_CUDA;
        ctx->own_stream = true;
    }
    if (cudaMalloc(&ctx->err_dev, 64) != cudaSuccess) return INSTA_ERR_CUDA;
    cudaMemset(ctx->err_dev, 0, 64);
    ctx->ray_counter = ctx->err_dev + 4;
    ctx->sample_counter = reinterpret_cast<unsigned long long*>(ctx->err_dev + 8);
    *out = ctx.release();
    return INSTA_OK;
}

int insta_ctx_destroy(insta_ctx* ctx) {
    if (!ctx) return INSTA_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->side) {
        cudaStreamSynchronize(ctx->side);
        cudaStreamDestroy(ctx->side);
    }
    if (ctx->side_mark) cudaEventDestroy(ctx->side_mark);
    if (ctx->copy) {
        cudaStreamSynchronize(ctx->copy);
        cudaStreamDestroy(ctx->copy);
        for (int k = 0; k < 2; ++k) {
            cudaEventDestroy(ctx->async_free[k]);
            ctx->release(ctx->async_rgba[k]);
            ctx->release(ctx->async_depth[k]);
        }
        cudaEventDestroy(ctx->async_done);
    }
    if (ctx->blas) cublasDestroy(ctx->blas);
    ctx->release(ctx->train_scratch);
    ctx->release(ctx->loss_scratch);
    ctx->release(ctx->train_t);
    if (ctx->loop_exec) cudaGraphExecDestroy(ctx->loop_exec);
    if (ctx->loop_graph) cudaGraphDestroy(ctx->loop_graph);
    if (ctx->loop_state) cudaFree(ctx->loop_state);
    if (ctx->capture) cudaStreamDestroy(ctx->capture);
    if (ctx->walk_stats) cudaFree(ctx->walk_stats);
    ctx->release(ctx->side_scratch);
    for (auto& kv : ctx->avatars)
        for (auto& f : kv.second->frames)
            if (f.second.ready) cudaEventDestroy(f.second.ready);
    for (auto& kv : ctx->avatars) {
        Avatar& a = *kv.second;
        for (DevBuf* b : {&a.faces, &a.mask, &a.adjacency, &a.canon_verts, &a.canon_area, &a.canon_frames, &a.frame_table,
                          &a.field.params, &a.field.image, &a.density_grid, &a.field.w32, &a.field.adam_m, &a.field.adam_v, &a.field.adam_steps, &a.field.w16, &a.field.ema, &a.field.train_params,
                          &a.field.train_image, &a.field.w16_train})
            ctx->release(*b);
        for (auto& f : a.frames)
            for (DevBuf* b : {&f.second.verts, &f.second.frames, &f.second.leaf_tris, &f.second.nodes, &f.second.bitfield})
                ctx->release(*b);
    }
    for (DevBuf* b : {&ctx->out_rgba, &ctx->out_depth, &ctx->extra, &ctx->bvh_scratch, &ctx->frame_jobs, &ctx->density_scratch,
                      &ctx->density_stage, &ctx->map_scratch, &ctx->grid_coords, &ctx->grid_idx, &ctx->grid_tmp})
        ctx->release(*b);
    Wave& w = ctx->wave;
    for (int b = 0; b < 2; ++b)
        for (int k = 0; k < 4; ++k) ctx->release(w.rays[b][k]);
    for (DevBuf* b : {&w.n_round, &w.sample_index, &w.sample_ray, &w.sample_key, &w.sample_order, &w.sort_bins, &w.samples, &w.march_t, &w.tiles,
                      &w.aux, &w.out, &w.out_f32, &w.counters, &w.req_table, &w.req_meta, &w.init_meta})
        ctx->release(*b);
    if (ctx->host_counters) cudaFreeHost(ctx->host_counters);
    if (ctx->host_alive) cudaFreeHost(ctx->host_alive);
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    cudaFree(ctx->err_dev);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return INSTA_OK;
}

const char* insta_last_error(const insta_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int insta_sync(insta_ctx* ctx) {
    return guarded(ctx, [&] { ctx->check_device(); });
}

int insta_memory_used(const insta_ctx* ctx, uint64_t* bytes) {
    if (!ctx || !bytes) return INSTA_ERR_INVALID_ARG;
    *bytes = ctx->used;
    return INSTA_OK;
}

int insta_canonical_set(insta_ctx* ctx, int avatar, const float* verts, int n_verts, const int32_t* faces, int n_faces,
                        const uint32_t* mask) {
    return guarded(ctx, [&] {
        if (!verts || !faces || n_verts < 3 || n_faces < 1) fail(INSTA_ERR_INVALID_ARG, "empty mesh");
        if (n_faces > 16384) fail(INSTA_ERR_UNSUPPORTED, "n_faces %d > 16384 (single-CTA BVH build)", n_faces);
        Avatar& a = ctx->avatar(avatar, true);
        if (a.has_canon && (a.V != n_verts || a.F != n_faces)) fail(INSTA_ERR_INVALID_ARG, "topology change on avatar %d", avatar);
        std::vector<int32_t> hf((size_t)n_faces * 3);
        std::vector<float> hv((size_t)n_verts * 3);
        CK(cudaMemcpy(hf.data(), faces, hf.size() * 4, cudaMemcpyDefault));
        CK(cudaMemcpy(hv.data(), verts, hv.size() * 4, cudaMemcpyDefault));
        for (int32_t i : hf)
            if (i < 0 || i >= n_verts) fail(INSTA_ERR_INVALID_ARG, "face index %d out of range", i);
        std::vector<uint32_t> hm((size_t)n_faces, 15u);
        if (mask) CK(cudaMemcpy(hm.data(), mask, hm.size() * 4, cudaMemcpyDefault));
        a.V = n_verts;
        a.F = n_faces;
        // TinyMesh::load (src/tiny_mesh.cu:62-86): centroid = float sum of the vertices / V
        float cs[3] = {0.f, 0.f, 0.f};
        for (int v = 0; v < n_verts; ++v)
            for (int k = 0; k < 3; ++k) cs[k] += hv[(size_t)v * 3 + k];
        for (int k = 0; k < 3; ++k) a.center[k] = cs[k] / (float)n_verts;
        std::vector<int32_t> adj = triangle_neighbours(hf, n_faces, n_verts);
        ctx->alloc(a.faces, hf.size() * 4);
        ctx->alloc(a.mask, hm.size() * 4);
        ctx->alloc(a.adjacency, adj.size() * 4);
        ctx->alloc(a.canon_verts, hv.size() * 4);
        ctx->alloc(a.canon_area, (size_t)n_faces * 4);
        ctx->alloc(a.canon_frames, (size_t)n_faces * sizeof(TriFrame));
        host_copy(a.faces.p, hf.data(), hf.size() * 4, ctx->stream);
        host_copy(a.mask.p, hm.data(), hm.size() * 4, ctx->stream);
        host_copy(a.adjacency.p, adj.data(), adj.size() * 4, ctx->stream);
        host_copy(a.canon_verts.p, hv.data(), hv.size() * 4, ctx->stream);
        CK(launch_tri_frames(n_faces, (const float*)a.canon_verts.p, (const int32_t*)a.faces.p, (const uint32_t*)a.mask.p, nullptr,
                             (float*)a.canon_area.p, (TriFrame*)a.canon_frames.p, 0, ctx->stream));
        // TinyMesh::build_triangles render box: vertex AABB inflated by 0.15 x |diag| (src/tiny_mesh.cu:157-162)
        float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int v = 0; v < n_verts; ++v)
            for (int k = 0; k < 3; ++k) { mn[k] = std::min(mn[k], hv[v * 3 + k]); mx[k] = std::max(mx[k], hv[v * 3 + k]); }
        float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
        float infl = sqrtf(dx * dx + (dy * dy + dz * dz)) * 0.15f;
        for (int k = 0; k < 3; ++k) { a.render_min[k] = mn[k] - infl; a.render_max[k] = mx[k] + infl; }
        a.has_canon = true;
        CK(cudaStreamSynchronize(ctx->stream));
    });
}

int insta_avatar_set_boxes(insta_ctx* ctx, int avatar, const float* train_min, const float* train_max, const float* render_min,
                           const float* render_max) {
    return guarded(ctx, [&] {
        Avatar& a = ctx->avatar(avatar);
        if (train_min) std::memcpy(a.train_min, train_min, 12);
        if (train_max) std::memcpy(a.train_max, train_max, 12);
        if (render_min) std::memcpy(a.render_min, render_min, 12);
        if (render_max) std::memcpy(a.render_max, render_max, 12);
        for (int k = 0; k < 3; ++k)
            if (!(a.train_max[k] > a.train_min[k])) fail(INSTA_ERR_INVALID_ARG, "empty train box");
    });
}

int insta_avatar_set_flags(insta_ctx* ctx, int avatar, uint32_t flags) {
    return guarded(ctx, [&] { ctx->avatar(avatar).flags = flags; });
}

int insta_frame_upload(insta_ctx* ctx, int avatar, int frame, const float* verts) {
    return guarded(ctx, [&] {
        Avatar& a = ctx->avatar(avatar);
        if (!verts || frame < 0) fail(INSTA_ERR_INVALID_ARG, "bad frame upload");
        ctx->alloc(ctx->bvh_scratch, bvh_scratch_bytes(a.F));
        Frame& f = prepare_frame(ctx, a, frame, verts);
        Stage st(ctx, INSTA_STAGE_FRAME, 3);
        CK(launch_tri_frames(a.F, (const float*)f.verts.p, (const int32_t*)a.faces.p, (const uint32_t*)a.mask.p,
                             (const float*)a.canon_area.p, nullptr, (TriFrame*)f.frames.p, 1, ctx->stream));
        CK(launch_bvh_build(f.view, (const float*)f.verts.p, (const int32_t*)a.faces.p, ctx->bvh_scratch.p, ctx->stream));
    });
}

int insta_frame_upload_batch(insta_ctx* ctx, int avatar, const int32_t* frames, int n, const float* const* verts) {
    return guarded(ctx, [&] {
        Avatar& a = ctx->avatar(avatar);
        if (n < 0 || (n > 0 && (!frames || !verts))) fail(INSTA_ERR_INVALID_ARG, "bad frame batch");
        if (n == 0) return;
        std::set<int> seen;
        for (int i = 0; i < n; ++i) {
            if (frames[i] < 0 || !verts[i]) fail(INSTA_ERR_INVALID_ARG, "bad frame %d in batch", i);
            if (!seen.insert(frames[i]).second) fail(INSTA_ERR_INVALID_ARG, "frame %d appears twice in the batch", frames[i]);
        }
        ctx->alloc(ctx->bvh_scratch, (size_t)n * bvh_scratch_bytes(a.F));
        ctx->alloc(ctx->frame_jobs, frame_batch_table_bytes(n));
        std::vector<FrameView> views((size_t)n);
        std::vector<const float*> dverts((size_t)n);
        for (int i = 0; i < n; ++i) {
            Frame& f = prepare_frame(ctx, a, frames[i], verts[i]);
            views[(size_t)i] = f.view;
            dverts[(size_t)i] = (const float*)f.verts.p;
        }
        Stage st(ctx, INSTA_STAGE_FRAME, 3);
        CK(launch_frames_batch(n, a.F, views.data(), dverts.data(), (const int32_t*)a.faces.p, (const uint32_t*)a.mask.p,
                               (const float*)a.canon_area.p, ctx->bvh_scratch.p, ctx->frame_jobs.p, ctx->stream));
    });
}

int insta_frame_upload_async(insta_ctx* ctx, int avatar, int frame, const float* verts, double occupancy_radius) {
    return guarded(ctx, [&] {
        Avatar& a = ctx->avatar(avatar);
        if (!verts || frame < 0) fail(INSTA_ERR_INVALID_ARG, "bad frame upload");
        if (occupancy_radius < 0.0) fail(INSTA_ERR_INVALID_ARG, "radius must be >= 0");
        if (!ctx->side) {
            CK(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&ctx->side_mark, cudaEventDisableTiming));
        }
        // after everything already queued on the context's stream (renders still reading this frame)
        CK(cudaEventRecord(ctx->side_mark, ctx->stream));
        CK(cudaStreamWaitEvent(ctx->side, ctx->side_mark, 0));
        ctx->alloc(ctx->side_scratch, bvh_scratch_bytes(a.F));
        Frame& f = prepare_frame(ctx, a, frame, verts, ctx->side);
        CK(launch_tri_frames(a.F, (const float*)f.verts.p, (const int32_t*)a.faces.p, (const uint32_t*)a.mask.p,
                             (const float*)a.canon_area.p, nullptr, (TriFrame*)f.frames.p, 1, ctx->side));
        CK(launch_bvh_build(f.view, (const float*)f.verts.p, (const int32_t*)a.faces.p, ctx->side_scratch.p, ctx->side));
        ctx->launches += 3;
        if (occupancy_radius > 0.0) {
            ctx->alloc(f.bitfield, (size_t)8 * GRID3 / 8);
            CK(launch_occupancy(f.view, occupancy_radius, (uint8_t*)f.bitfield.p, ctx->err_dev, ctx->side));
            ctx->launches += 1;
            f.has_occupancy = true;
        }
        if (!f.ready) CK(cudaEventCreateWithFlags(&f.ready, cudaEventDisableTiming));
        CK(cudaEventRecord(f.ready, ctx->side));
        f.pending = true;
    });
}

int insta_frame_wait(insta_ctx* ctx, int avatar, int frame) {
    return guarded(ctx, [&] { use_frame(ctx, ctx->avatar(avatar), frame); });
}

int insta_frame_release(insta_ctx* ctx, int avatar, int frame) {
    return guarded(ctx, [&] {
        Avatar& a = ctx->avatar(avatar);
        auto it = a.frames.find(frame);
        if (it == a.frames.end()) return;
        CK(cudaStreamSynchronize(ctx->stream));
        if (it->second.ready) {
            CK(cudaEventSynchronize(it->second.ready));
            cudaEventDestroy(it->second.ready);
        }
        for (DevBuf* b : {&it->second.verts, &it->second.frames, &it->second.leaf_tris, &it->second.nodes, &it->second.bitfield})
            ctx->release(*b);
        a.frames.erase(it);
        a.table_dirty = true;
    });
}

int insta_occupancy_from_mesh(insta_ctx* ctx, int avatar, int frame, double radius) {
    return guarded(ctx, [&] {
        if (!(radius > 0.0)) fail(INSTA_ERR_INVALID_ARG, "radius must be positive");
        Avatar& a = ctx->avatar(avatar);
        Frame& f = use_frame(ctx, a, frame);
        ctx->alloc(f.bitfield, (size_t)8 * GRID3 / 8);
        Stage st(ctx, INSTA_STAGE_OCCUPANCY, 1);
        CK(launch_occupancy(f.view, radius, (uint8_t*)f.bitfield.p, ctx->err_dev, ctx->stream));
        f.has_occupancy = true;
    });
}

int insta_occupancy_set(insta_ctx* ctx, int avatar, int frame, const uint8_t* bits) {
    return guarded(ctx, [&] {
        if (!bits) fail(INSTA_ERR_INVALID_ARG, "null bitfield");
        Frame& f = use_frame(ctx, ctx->avatar(avatar), frame);
        ctx->alloc(f.bitfield, (size_t)8 * GRID3 / 8);
        host_copy(f.bitfield.p, bits, (size_t)8 * GRID3 / 8, ctx->stream);
        f.has_occupancy = true;
    });
}

int insta_density_grid_load(insta_ctx* ctx, int avatar, int frame, const void* grid, uint32_t n_cascades, int fp16) {
    return guarded(ctx, [&] {
        if (!grid) fail(INSTA_ERR_INVALID_ARG, "null density grid");
        if (n_cascades < 1 || n_cascades > 8) fail(INSTA_ERR_INVALID_ARG, "n_cascades must be 1..8, got %u", n_cascades);
        Frame& f = use_frame(ctx, ctx->avatar(avatar), frame);
        ctx->alloc(f.bitfield, (size_t)8 * GRID3 / 8);
        ctx->alloc(ctx->density_scratch, density_scratch_bytes(n_cascades));
        const void* src = grid;
        if (fp16 && !is_device_ptr(grid)) {
            ctx->alloc(ctx->density_stage, (size_t)n_cascades * GRID3 * 2);
            host_copy(ctx->density_stage.p, grid, (size_t)n_cascades * GRID3 * 2, ctx->stream);
            src = ctx->density_stage.p;
        }
        Stage st(ctx, INSTA_STAGE_OCCUPANCY, fp16 ? 11 : 10);
        CK(launch_density_grid(src, fp16, n_cascades, ctx->density_scratch.p, (uint8_t*)f.bitfield.p, ctx->stream));
        f.has_occupancy = true;
    });
}

int insta_density_grid_reset(insta_ctx* ctx, int avatar, const float* grid, uint32_t n_cascades) {
    return guarded(ctx, [&] {
        if (n_cascades < 1 || n_cascades > 8) fail(INSTA_ERR_INVALID_ARG, "n_cascades must be 1..8, got %u", n_cascades);
        Avatar& a = ctx->avatar(avatar);
        const size_t bytes = (size_t)n_cascades * GRID3 * sizeof(float);
        ctx->alloc(a.density_grid, bytes);
        a.grid_cascades = n_cascades;
        if (grid) host_copy(a.density_grid.p, grid, bytes, ctx->stream);
        else CK(cudaMemsetAsync(a.density_grid.p, 0, bytes, ctx->stream));
    });
}

int insta_density_grid_read(insta_ctx* ctx, int avatar, float* out) {
    return guarded(ctx, [&] {
        if (!out) fail(INSTA_ERR_INVALID_ARG, "null output");
        Avatar& a = ctx->avatar(avatar);
        if (!a.density_grid.p) fail(INSTA_ERR_NOT_READY, "avatar %d has no density grid (insta_density_grid_reset)", avatar);
        host_copy(out, a.density_grid.p, (size_t)a.grid_cascades * GRID3 * sizeof(float), ctx->stream);
        ctx->check_device();
    });
}

int insta_density_grid_update(insta_ctx* ctx, int avatar, insta_density_update_desc* d) {
    return guarded(ctx, [&] {
        if (!d) fail(INSTA_ERR_INVALID_ARG, "null description");
        Avatar& a = ctx->avatar(avatar);
        if (!a.field.ready) fail(INSTA_ERR_NOT_READY, "avatar %d has no field parameters", avatar);
        if (!a.density_grid.p) fail(INSTA_ERR_NOT_READY, "avatar %d has no density grid (insta_density_grid_reset)", avatar);
        if (d->n_cascades != a.grid_cascades)
            fail(INSTA_ERR_INVALID_ARG, "n_cascades %u differs from the grid's %u", d->n_cascades, a.grid_cascades);
        const uint64_t n64 = (uint64_t)d->n_uniform + d->n_nonuniform;
        if (n64 == 0 || n64 >= (1ull << 30)) fail(INSTA_ERR_INVALID_ARG, "sample count must be 1 .. 2^30 - 1, got %llu", (unsigned long long)n64);
        if (d->n_frames < 1) fail(INSTA_ERR_INVALID_ARG, "n_frames must be >= 1");
        for (int k = 0; k < d->n_frames; ++k)
            if (!a.frames.count(k)) fail(INSTA_ERR_NOT_READY, "frame %d (of the %d the warp picks from) is not uploaded", k, d->n_frames);
        const uint32_t n = (uint32_t)n64, stride = 11;
        refresh_frame_table(ctx, a);
        wait_all_frames(ctx, a);
        ctx->alloc(ctx->grid_coords, (size_t)n * stride * sizeof(float));
        ctx->alloc(ctx->grid_idx, (size_t)n * sizeof(uint32_t));
        ctx->alloc(ctx->grid_tmp, (size_t)d->n_cascades * GRID3 * sizeof(float));
        float* coords = (float*)ctx->grid_coords.p;
        uint32_t* idx = (uint32_t*)ctx->grid_idx.p;
        const TilePlan& P = a.field.plan;
        const uint64_t tiles = ((uint64_t)n + 127) / 128;
        Wave& w = ctx->wave;
        ctx->alloc(w.tiles, tiles * P.tile_bytes);
        ctx->alloc(w.out, tiles * 128 * sizeof(uint2));
        ctx->alloc(w.out_f32, tiles * 128 * sizeof(float4));
        {
            Stage st(ctx, INSTA_STAGE_OCCUPANCY, (uint32_t)d->n_frames <= kMaxRequests ? 11 : 6);
            CK(cudaMemsetAsync(ctx->grid_tmp.p, 0, (size_t)d->n_cascades * GRID3 * sizeof(float), ctx->stream));
            CK(launch_grid_samples(d->n_uniform, d->n_nonuniform, d->grid_rng.state, d->grid_rng.inc, d->ema_step, d->aabb_min, d->aabb_max,
                                   (const float*)a.density_grid.p, d->n_cascades, coords, stride, idx, ctx->stream));
            if ((uint32_t)d->n_frames <= kMaxRequests) {
                // the sample domain: cascade c spans 0.5 -+ 2^(c-1) of the unit cube, relative to the box
                const float half = 0.5f * (float)(1u << (d->n_cascades - 1));
                float lo[3], hi[3];
                for (int k = 0; k < 3; ++k) {
                    const float ext = d->aabb_max[k] - d->aabb_min[k];
                    lo[k] = (0.5f - half - d->aabb_min[k]) / ext;
                    hi[k] = (0.5f + half - d->aabb_min[k]) / ext;
                }
                ctx->alloc(ctx->map_scratch, warp_sorted_scratch_bytes(n, (uint32_t)d->n_frames));
                CK(launch_warp_random_sorted((const FrameView*)a.frame_table.p, (uint32_t)d->n_frames, deform_view(a), coords, stride, n,
                                             d->warp_rng.state, d->warp_rng.inc, lo, hi, ctx->map_scratch.p, ctx->err_dev, ctx->stream));
            } else {
                CK(launch_warp_random((const FrameView*)a.frame_table.p, (uint32_t)d->n_frames, deform_view(a), coords, stride, n,
                                      d->warp_rng.state, d->warp_rng.inc, ctx->err_dev, ctx->stream));
            }
            if (d->debug_pos)
                CK(cudaMemcpy2DAsync(d->debug_pos, 3 * sizeof(float), coords, stride * sizeof(float), 3 * sizeof(float), n,
                                     cudaMemcpyDefault, ctx->stream));
            if (d->debug_idx) CK(cudaMemcpyAsync(d->debug_idx, idx, (size_t)n * sizeof(uint32_t), cudaMemcpyDefault, ctx->stream));
            CK(cudaMemsetAsync(w.tiles.p, 0, tiles * P.tile_bytes, ctx->stream));
            // a field with expression dims gets 1 in each of them (NerfNetwork::density,
            // NGP/nerf_network.h:107-127,401-410: the per-sample random code is disabled there)
            CK(launch_encode_coords(a.field.view, coords, stride, n, (uint8_t*)w.tiles.p, P.tile_bytes, P.k_in, ctx->stream, true));
            MlpArgs m{};
            m.fv = a.field.view; m.plan = P; m.tiles = (const uint8_t*)w.tiles.p; m.n_alive = nullptr; m.n_samples = n;
            m.out = (uint2*)w.out.p; m.out_f32 = (float4*)w.out_f32.p; m.err = ctx->err_dev;
            CK(launch_mlp(m, (uint32_t)tiles, ctx->stream));
            CK(launch_splat_ema(n, idx, (const uint2*)w.out.p, (const float4*)w.out_f32.p, a.field.view.precision != 0,
                                (float*)ctx->grid_tmp.p, (float*)a.density_grid.p, d->n_cascades * GRID3, d->decay, ctx->stream));
        }
        if (d->bitfield_frame >= 0) {
            Frame& f = use_frame(ctx, a, d->bitfield_frame);
            ctx->alloc(f.bitfield, (size_t)8 * GRID3 / 8);
            ctx->alloc(ctx->density_scratch, density_scratch_bytes(d->n_cascades));
            Stage st(ctx, INSTA_STAGE_OCCUPANCY, 10);
            CK(launch_density_grid(a.density_grid.p, 0, d->n_cascades, ctx->density_scratch.p, (uint8_t*)f.bitfield.p, ctx->stream));
            f.has_occupancy = true;
        }
        // the reference's host-side bookkeeping after the update: ++density_grid_ema_step and
        // density_grid_rng.advance() with pcg32's default jump of 2^32
        d->ema_step += 1;
        Pcg32 r{d->grid_rng.state, d->grid_rng.inc};
        r.advance((int64_t)1 << 32);
        d->grid_rng.state = r.state;
    });
}

int insta_occupancy_get(insta_ctx* ctx, int avatar, int frame, uint8_t* bits) {
    return guarded(ctx, [&] {
        if (!bits) fail(INSTA_ERR_INVALID_ARG, "null bitfield");
        Frame& f = use_frame(ctx, ctx->avatar(avatar), frame);
        if (!f.has_occupancy) fail(INSTA_ERR_NOT_READY, "frame %d has no occupancy", frame);
        host_copy(bits, f.bitfield.p, (size_t)8 * GRID3 / 8, ctx->stream);
        ctx->check_device();
    });
}

int insta_canonical_map(insta_ctx* ctx, int avatar, int frame, float* coords, uint32_t stride, uint32_t n_extra, int64_t n) {
    return guarded(ctx, [&] {
        if (n < 0 || (n > 0 && !coords)) fail(INSTA_ERR_INVALID_ARG, "bad coordinate buffer");
        if (stride < 11 + n_extra) fail(INSTA_ERR_INVALID_ARG, "stride %u < 11 + n_extra", stride);
        Avatar& a = ctx->avatar(avatar);
        if (n == 0) return;
        refresh_frame_table(ctx, a);
        if (frame >= 0) use_frame(ctx, a, frame); else wait_all_frames(ctx, a);
        const bool sorted = n >= kMapSortedMin && n < ((int64_t)1 << 30) && (frame >= 0 || a.table_frames <= kMaxRequests);
        if (sorted) {
            // render_deformed (fixed frame) sorts by cell; surface_closest_point by (holder frame, cell)
            const uint32_t n_frames = frame >= 0 ? 1u : a.table_frames;
            const FrameView* frames = (const FrameView*)a.frame_table.p + (frame >= 0 ? frame : 0);
            ctx->alloc(ctx->map_scratch, warp_sorted_scratch_bytes((uint32_t)n, n_frames));
            Stage st(ctx, INSTA_STAGE_CANONICAL_MAP, 6);
            CK(launch_canonical_map_coords_sorted(frames, n_frames, frame >= 0, deform_view(a), coords, stride, n_extra, (uint32_t)n,
                                                  ctx->map_scratch.p, ctx->err_dev, ctx->stream));
        } else {
            Stage st(ctx, INSTA_STAGE_CANONICAL_MAP, 1);
            CK(launch_canonical_map_coords((const FrameView*)a.frame_table.p, a.table_frames, deform_view(a), coords, stride, n_extra, n,
                                           frame, ctx->err_dev, ctx->stream));
        }
    });
}

int insta_training_samples(insta_ctx* ctx, int avatar, int grid_frame, const float* rays, const uint32_t* image,
                           const float* start_rand, const float* extra, uint32_t n_images, int64_t n_rays, float cone_angle,
                           uint32_t max_samples, float* coords, uint32_t stride, uint32_t* ray_indices, uint32_t* numsteps,
                           uint32_t* counters) {
    return guarded(ctx, [&] {
        if (n_rays < 0 || (n_rays > 0 && (!rays || !image || !start_rand)) || !coords || !ray_indices || !numsteps || !counters)
            fail(INSTA_ERR_INVALID_ARG, "null buffer");
        if (stride < 11) fail(INSTA_ERR_INVALID_ARG, "stride %u < 11", stride);
        if (max_samples >= (1u << 30)) fail(INSTA_ERR_INVALID_ARG, "max_samples must be below 2^30");
        if (!(cone_angle >= 0.f)) fail(INSTA_ERR_INVALID_ARG, "cone_angle must be >= 0");
        for (const void* p : {(const void*)rays, (const void*)image, (const void*)start_rand, (const void*)coords, (const void*)ray_indices,
                              (const void*)numsteps, (const void*)counters})
            if (n_rays > 0 && !is_device_ptr(p)) fail(INSTA_ERR_INVALID_ARG, "insta_training_samples takes device pointers");
        Avatar& a = ctx->avatar(avatar);
        Frame& g = use_frame(ctx, a, grid_frame);
        if (!g.has_occupancy) fail(INSTA_ERR_NOT_READY, "frame %d has no occupancy bitfield", grid_frame);
        refresh_frame_table(ctx, a);
        wait_all_frames(ctx, a);   // the warp picks each record's frame
        CK(cudaMemsetAsync(counters, 0, 2 * sizeof(uint32_t), ctx->stream));
        if (n_rays == 0) return;
        TrainArgs T{};
        T.rays = rays; T.image = image; T.start_rand = start_rand; T.extra = extra;
        T.n_extra = stride - 11; T.n_images = n_images; T.n_rays = n_rays;
        for (int k = 0; k < 3; ++k) { T.aabb_min[k] = a.train_min[k]; T.aabb_max[k] = a.train_max[k]; }
        T.cone_angle = cone_angle; T.max_samples = max_samples; T.bitfield = (const uint8_t*)g.bitfield.p;
        T.coords = coords; T.stride = stride; T.ray_indices = ray_indices; T.numsteps = numsteps; T.counters = counters;
        float* tbuf = nullptr;
        if (n_rays <= kTrainMarchOnceMaxRays) {
            ctx->alloc(ctx->train_t, (size_t)n_rays * 1024 * 4);
            tbuf = (float*)ctx->train_t.p;
        }
        { Stage st(ctx, INSTA_STAGE_MARCH, tbuf ? 2 : 1); CK(launch_training_samples(T, tbuf, ctx->stream)); }
        // the warp with per-record frames (surface_closest_point, testbed_nerf.cu:3290): large sample
        // buffers take the (frame, cell)-sorted warp walk over the records the march wrote
        if (max_samples >= kMapSortedMin && a.table_frames <= kMaxRequests) {
            ctx->alloc(ctx->map_scratch, warp_sorted_scratch_bytes(max_samples, a.table_frames));
            Stage st(ctx, INSTA_STAGE_CANONICAL_MAP, 6);
            CK(launch_canonical_map_coords_sorted((const FrameView*)a.frame_table.p, a.table_frames, 0, deform_view(a), coords, stride,
                                                  stride - 11, max_samples, ctx->map_scratch.p, ctx->err_dev, ctx->stream, counters + 1));
        } else {
            Stage st(ctx, INSTA_STAGE_CANONICAL_MAP, 1);
            CK(launch_canonical_map_coords((const FrameView*)a.frame_table.p, a.table_frames, deform_view(a), coords, stride, stride - 11,
                                           (int64_t)max_samples, -1, ctx->err_dev, ctx->stream, counters + 1));
        }
    });
}

int insta_canonical_map_soa(insta_ctx* ctx, int avatar, int frame, const float* pts, int64_t n, int32_t* out_idx, float* out_canon) {
    return guarded(ctx, [&] {
        if (n < 0 || (n > 0 && (!pts || !out_idx || !out_canon))) fail(INSTA_ERR_INVALID_ARG, "bad buffers");
        Avatar& a = ctx->avatar(avatar);
        Frame& f = use_frame(ctx, a, frame);
        if (n >= kMapSortedMin && n < ((int64_t)1 << 31)) {
            ctx->alloc(ctx->map_scratch, map_sorted_scratch_bytes(n));
            Stage st(ctx, INSTA_STAGE_CANONICAL_MAP, 6);
            CK(launch_canonical_map_sorted(f.view, deform_view(a), pts, n, out_idx, out_canon, ctx->map_scratch.p, ctx->err_dev,
                                           ctx->stream));
        } else {
            Stage st(ctx, INSTA_STAGE_CANONICAL_MAP, 1);
            CK(launch_canonical_map_soa(f.view, deform_view(a), pts, n, out_idx, out_canon, ctx->err_dev, ctx->stream));
        }
    });
}

int insta_field_param_count(const insta_field_desc* desc, uint64_t* n_params) {
    if (!desc || !n_params) return INSTA_ERR_INVALID_ARG;
    try {
        *n_params = field_layout(*desc).total;
        return INSTA_OK;
    } catch (const Failure& e) {
        return e.code;
    }
}

int insta_params_load(insta_ctx* ctx, int avatar, const insta_field_desc* desc, const uint16_t* params, uint64_t n_params) {
    return guarded(ctx, [&] {
        if (!desc || !params) fail(INSTA_ERR_INVALID_ARG, "null field description or parameters");
        Avatar& a = ctx->avatar(avatar, true);
        FieldLayout L = field_layout(*desc);
        if (n_params != L.total) fail(INSTA_ERR_INVALID_ARG, "expected %llu parameters, got %llu", (unsigned long long)L.total,
                                      (unsigned long long)n_params);
        Field& fd = a.field;
        fd.desc = *desc;
        fd.n_params = n_params;
        if (!ctx->keep_master) {
            fd.w32_valid = false;
            fd.adam_step = 0;
            fd.ema_step = 0;
            fd.train_valid = false;
        }
        ctx->alloc(fd.params, n_params * 2);
        host_copy(fd.params.p, params, n_params * 2, ctx->stream);
        // MLP weight image in the tensor-core operand layout (umma.cuh), one B tile per operand
        std::vector<uint16_t> mlp(L.table_off);
        CK(cudaMemcpyAsync(mlp.data(), params, L.table_off * 2, cudaMemcpyDefault, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        TilePlan plan{};
        uint32_t off = 0;
        std::vector<uint8_t> image;
        // copy columns [k0, k0 + K) of layer l ([N][Kin] row-major) into a [N][K] operand tile
        auto add_tile = [&](int l, uint32_t k0, uint32_t K) -> uint32_t {
            const uint32_t N = L.layer_n[l], Kin = L.layer_k[l];
            const uint32_t at = off;
            image.resize(off + (size_t)N * K * 2, 0);
            for (uint32_t n = 0; n < N; ++n)
                for (uint32_t k = 0; k < K && k0 + k < Kin; ++k) {
                    uint16_t w = mlp[L.layer_off[l] + (uint64_t)n * Kin + k0 + k];
                    if (desc->precision == INSTA_PRECISION_BF16) w = half_to_bf16_bits(w);
                    std::memcpy(&image[at + tile_offset(n, k, K)], &w, 2);
                }
            off = (off + N * K * 2 + 127) / 128 * 128;
            return at;
        };
        // FP8: one byte per weight, scaled per layer by s = max|W| / 448
        const bool fp8 = desc->precision == INSTA_PRECISION_FP8;
        float lscale[8] = {1.f, 1.f, 1.f, 1.f, 1.f, 1.f, 1.f, 1.f};
        if (fp8)
            for (int l = 0; l < L.n_density + L.n_rgb; ++l) {
                float mx = 0.f;
                for (uint64_t i = 0; i < (uint64_t)L.layer_n[l] * L.layer_k[l]; ++i)
                    mx = std::max(mx, std::fabs(half_to_float(mlp[L.layer_off[l] + i])));
                lscale[l] = mx > 0.f ? mx / 448.0f : 1.0f;
            }
        auto add_tile8 = [&](int l, uint32_t k0, uint32_t K) -> uint32_t {
            const uint32_t N = L.layer_n[l], Kin = L.layer_k[l];
            const uint32_t at = off;
            image.resize(off + (size_t)N * K, 0);
            for (uint32_t n = 0; n < N; ++n)
                for (uint32_t k = 0; k < K && k0 + k < Kin; ++k)
                    image[at + tile_offset8(n, k, K)] = float_to_e4m3(half_to_float(mlp[L.layer_off[l] + (uint64_t)n * Kin + k0 + k]) / lscale[l]);
            off = (off + N * K + 127) / 128 * 128;
            return at;
        };
        plan.k_in = (L.layer_k[0] + 15) / 16 * 16;
        plan.k8 = (L.layer_k[0] + 31) / 32 * 32;
        // the E4M3 density input rows of the per-CTA kernel take one 16 KiB buffer: 128 B per row
        if (fp8 && plan.k8 > 128) fail(INSTA_ERR_UNSUPPORTED, "FP8 fields take at most 128 density inputs (got %u)", L.layer_k[0]);
        plan.n_dh = (uint32_t)L.n_density - 1;
        const int r0 = L.n_density;
        plan.n_rh = (uint32_t)L.n_rgb - 1;
        if (fp8) {
            for (uint32_t l = 0; l < plan.n_dh; ++l) plan.d_off[l] = add_tile8((int)l, 0, l == 0 ? plan.k8 : 64);
            plan.d_out = add_tile8(L.n_density - 1, 0, 64);
            plan.r0_dens = plan.r0_sh = add_tile8(r0, 0, 32);   // [density out | SH] as one K = 32 operand
            for (uint32_t l = 1; l < plan.n_rh; ++l) plan.r_off[l] = add_tile8(r0 + (int)l, 0, 64);
            plan.r_out = add_tile8(r0 + L.n_rgb - 1, 0, 64);
            // the scales travel with the weights (a batch may mix avatars)
            plan.scales = off;
            image.resize(off + sizeof(lscale), 0);
            std::memcpy(&image[off], lscale, sizeof(lscale));
            off = (off + (uint32_t)sizeof(lscale) + 127) / 128 * 128;
        } else {
            for (uint32_t l = 0; l < plan.n_dh; ++l) plan.d_off[l] = add_tile((int)l, 0, l == 0 ? plan.k_in : 64);
            plan.d_out = add_tile(L.n_density - 1, 0, 64);
            plan.r0_dens = add_tile(r0, 0, 16);
            plan.r0_sh = add_tile(r0, 16, 16);
            for (uint32_t l = 1; l < plan.n_rh; ++l) plan.r_off[l] = add_tile(r0 + (int)l, 0, 64);
            plan.r_out = add_tile(r0 + L.n_rgb - 1, 0, 64);
        }
        plan.bytes = off;
        plan.tile_bytes = hash_tile_bytes(plan.k_in) + sh_tile_bytes();
        if (plan.bytes > 64 * 1024) fail(INSTA_ERR_UNSUPPORTED, "MLP weights exceed 64 KiB of shared memory");
        ctx->alloc(fd.image, image.size());
        CK(cudaMemcpyAsync(fd.image.p, image.data(), image.size(), cudaMemcpyHostToDevice, ctx->stream));
        fd.plan = plan;
        FieldView& v = fd.view;
        std::memset(&v, 0, sizeof(v));
        v.table = static_cast<const uint16_t*>(fd.params.p) + L.table_off;
        v.mlp_smem = static_cast<const uint8_t*>(fd.image.p);
        v.mlp_smem_bytes = plan.bytes;
        v.n_levels = desc->n_levels;
        v.n_features = desc->n_features_per_level;
        v.n_extra = desc->n_extra_dims;
        for (uint32_t l = 0; l < desc->n_levels; ++l) {
            v.level_scale[l] = L.lvl_scale[l];
            v.level_res[l] = L.lvl_res[l];
            v.level_size[l] = L.lvl_size[l];
            v.level_off[l] = (uint32_t)L.lvl_off[l];
            v.level_dense[l] = (uint64_t)L.lvl_res[l] * L.lvl_res[l] * L.lvl_res[l] <= L.lvl_size[l] ? 1 : 0;
        }
        v.precision = (int)desc->precision;
        CK(cudaStreamSynchronize(ctx->stream));
        fd.ready = true;
    });
}

namespace {
void field_eval_view(insta_ctx* ctx, int avatar, Avatar& a, const FieldView& fv, const float* coords, uint32_t stride, int64_t n,
                     float* out4) {
    if (!a.field.ready) fail(INSTA_ERR_NOT_READY, "avatar %d has no field parameters", avatar);
    if (n < 0 || (n > 0 && (!coords || !out4))) fail(INSTA_ERR_INVALID_ARG, "bad buffers");
    if (stride < 11 + a.field.desc.n_extra_dims) fail(INSTA_ERR_INVALID_ARG, "stride too small");
    if (n == 0) return;
    const TilePlan& P = a.field.plan;
    const uint64_t tiles = ((uint64_t)n + 127) / 128;
    Wave& w = ctx->wave;
    ctx->alloc(w.tiles, tiles * P.tile_bytes);
    ctx->alloc(w.out, tiles * 128 * sizeof(uint2));
    ctx->alloc(w.out_f32, tiles * 128 * sizeof(float4));
    CK(cudaMemsetAsync(w.tiles.p, 0, tiles * P.tile_bytes, ctx->stream));
    Stage st(ctx, INSTA_STAGE_FIELD, 3);
    CK(launch_encode_coords(fv, coords, stride, n, (uint8_t*)w.tiles.p, P.tile_bytes, P.k_in, ctx->stream));
    MlpArgs m{};
    m.fv = fv; m.plan = P; m.tiles = (const uint8_t*)w.tiles.p; m.n_alive = nullptr; m.n_samples = n;
    m.out = (uint2*)w.out.p; m.out_f32 = (float4*)w.out_f32.p; m.err = ctx->err_dev;
    CK(launch_mlp(m, (uint32_t)tiles, ctx->stream));
    CK(launch_unpack((const uint2*)w.out.p, (const float4*)w.out_f32.p, fv.precision != 0, n, (float4*)out4, ctx->stream));
}
}  // namespace

int insta_field_eval(insta_ctx* ctx, int avatar, const float* coords, uint32_t stride, int64_t n, float* out4) {
    return guarded(ctx, [&] {
        Avatar& a = ctx->avatar(avatar);
        field_eval_view(ctx, avatar, a, a.field.view, coords, stride, n, out4);
    });
}

int insta_field_eval_training(insta_ctx* ctx, int avatar, const float* coords, uint32_t stride, int64_t n, float* out4) {
    return guarded(ctx, [&] {
        Avatar& a = ctx->avatar(avatar);
        field_eval_view(ctx, avatar, a, a.field.train_valid ? a.field.train_view : a.field.view, coords, stride, n, out4);
    });
}

namespace {
TrainShape train_shape(const Field& fd) {
    const FieldLayout L = field_layout(fd.desc);
    TrainShape t{};
    t.kd = L.layer_k[0];
    t.n_density = L.n_density;
    t.n_rgb = L.n_rgb;
    for (int l = 0; l < 8; ++l) t.layer_off[l] = L.layer_off[l];
    t.table_off = L.table_off;
    return t;
}

// The tcgen05 training plan of a field: weight-image tiles (forward B tiles, and W^T for the input
// gradients), TMEM columns of the weight-gradient accumulators (from column 96, 32-aligned), and
// the shared-memory layout.  False when the field does not fit one CTA (shared memory, TMEM).
bool train_mlp_plan(const FieldLayout& L, TrainMlpPlan& P, TrainImageList& I) {
    P = TrainMlpPlan{};
    I = TrainImageList{};
    const int nl = L.n_density + L.n_rgb;
    if (nl > 8 || L.n_density < 2 || L.n_rgb < 2) return false;
    P.n_density = (uint32_t)L.n_density;
    P.n_rgb = (uint32_t)L.n_rgb;
    P.kd = L.layer_k[0];
    if (P.kd % 16 || P.kd > 64) return false;
    uint32_t off = 0, col = 128;   // TMEM: columns 0..127 the two slots' working accumulators
    auto add = [&](uint32_t n, uint32_t k, uint64_t w_off, uint32_t rows, uint32_t cols, uint32_t tr) {
        TrainImageTile& T = I.tile[I.n_tiles++];
        T = TrainImageTile{off, n, k, w_off, rows, cols, 0u, 0u, tr};
        const uint32_t at = off;
        off = (off + n * k * 2 + 127) / 128 * 128;
        return at;
    };
    for (int l = 0; l < nl; ++l) {
        TrainMlpLayer& Y = P.layer[l];
        Y.n_out = L.layer_n[l];
        Y.n_in = L.layer_k[l];
        if (Y.n_in > 64 || (Y.n_out != 16 && Y.n_out != 64)) return false;
        if (l == L.n_density && Y.n_in != 32) return false;   // the colour input [density output | SH]
        Y.k_pad = (Y.n_in + 15) / 16 * 16;
        Y.w_off = L.layer_off[l];
        Y.n_out_real = l == nl - 1 ? 3u : Y.n_out;
        Y.fwd_img = add(Y.n_out, Y.k_pad, Y.w_off, Y.n_out, Y.n_in, 0);
        // only the density-output part of the colour input has a gradient to pass on
        Y.bwd_n = l == L.n_density ? 16u : Y.k_pad;
        Y.bwd_img = add(Y.bwd_n, Y.n_out, Y.w_off, Y.n_out, Y.n_in, 1);
        Y.dw_col = col;
        col = (col + Y.n_out + 31) / 32 * 32;
    }
    if (col > 512) return false;
    P.img_bytes = off;
    auto r1k = [](uint32_t b) { return (b + 1023u) & ~1023u; };
    uint32_t o = 1024;
    P.s_img = o; o = r1k(o + P.img_bytes);
    for (int s = 0; s < 2; ++s) {
        P.s_x[s] = o; o = r1k(o + 128 * P.kd * 2);
        P.s_rin[s] = o; o += 128 * 32 * 2;
        for (int k = 0; k < nl - 2; ++k) { P.s_kept[s][k] = o; o += 128 * 64 * 2; }
        P.s_dy[s] = o; o += 128 * 64 * 2;
    }
    o += 16384;   // tail
    P.smem_bytes = o;
    return o <= 227u * 1024u;
}

void ensure_master(insta_ctx* ctx, Field& fd) {
    if (fd.w32_valid) return;
    ctx->alloc(fd.w32, fd.n_params * 4);
    CK(launch_half_to_float(fd.n_params, fd.params.p, (float*)fd.w32.p, ctx->stream));
    fd.w32_valid = true;
}
}  // namespace

int insta_field_backward(insta_ctx* ctx, int avatar, const float* coords, uint32_t stride, int64_t n, const float* dl_dout, float* grad,
                         float* out4) {
    return insta_field_backward_ex(ctx, avatar, coords, stride, n, dl_dout, grad, out4, nullptr);
}

int insta_field_backward_ex(insta_ctx* ctx, int avatar, const float* coords, uint32_t stride, int64_t n, const float* dl_dout,
                            float* grad, float* out4, float* dl_dextra) {
    return guarded(ctx, [&] {
        Avatar& a = ctx->avatar(avatar);
        Field& fd = a.field;
        if (!fd.ready) fail(INSTA_ERR_NOT_READY, "avatar %d has no field parameters", avatar);
        if (n < 0 || n >= ((int64_t)1 << 24)) fail(INSTA_ERR_INVALID_ARG, "sample count must be 0 .. 2^24 - 1");
        if (n > 0 && (!coords || (!out4 && !(dl_dout && grad)))) fail(INSTA_ERR_INVALID_ARG, "bad buffers");
        if ((dl_dout == nullptr) != (grad == nullptr)) fail(INSTA_ERR_INVALID_ARG, "output gradients and parameter gradients go together");
        if (stride < 11 + fd.desc.n_extra_dims) fail(INSTA_ERR_INVALID_ARG, "stride too small");
        if ((uintptr_t)grad & 7) fail(INSTA_ERR_INVALID_ARG, "grad must be 8-byte aligned");   // paired table atomics
        if (fd.desc.n_features_per_level >= 4 && ((uintptr_t)grad & 15))
            fail(INSTA_ERR_INVALID_ARG, "grad must be 16-byte aligned for 4 or 8 features per level");   // 16-byte table atomics
        if (dl_dextra && !(dl_dout && grad)) fail(INSTA_ERR_INVALID_ARG, "dl_dextra needs the backward (dl_dout and grad)");
        if (n == 0) return;
        const int extra_k = (dl_dextra && fd.desc.n_extra_dims) ? 1 : 0;
        // the encode reads the FP16 copy of the training weights (under an Ema the field's own
        // parameters are the average)
        FieldView tv = fd.view;
        if (fd.train_valid) tv.table = fd.train_view.table;
        if (ctx->train_tc) {
            ensure_master(ctx, fd);
            const TrainShape t = train_shape(fd);
            TrainMlpPlan plan;
            TrainImageList images;
            if (!train_mlp_plan(field_layout(fd.desc), plan, images))
                fail(INSTA_ERR_UNSUPPORTED, "the field's MLPs do not fit the tcgen05 training kernel; use INSTA_TRAIN_MATH_TF32");
            ctx->alloc(ctx->train_images, plan.img_bytes);
            ctx->alloc(ctx->train_scratch, ((size_t)2 * t.kd + 32) * (size_t)n * 4);
            Stage st(ctx, INSTA_STAGE_TRAIN, ((dl_dout && grad) ? 4 : 3) + extra_k);
            CK(launch_field_train_tc(tv, t, plan, images, (uint8_t*)ctx->train_images.p, (const float*)fd.w32.p, coords, stride,
                                     (uint32_t)n, dl_dout, out4, grad, (float*)ctx->train_scratch.p, ctx->err_dev, ctx->stream, dl_dextra));
            return;
        }
        if (!ctx->blas) {
            if (cublasCreate(&ctx->blas) != CUBLAS_STATUS_SUCCESS) fail(INSTA_ERR_CUDA, "cublasCreate failed");
            if (cublasSetMathMode(ctx->blas, ctx->train_tf32 ? CUBLAS_TF32_TENSOR_OP_MATH : CUBLAS_DEFAULT_MATH) != CUBLAS_STATUS_SUCCESS)
                fail(INSTA_ERR_CUDA, "cublasSetMathMode failed");
        }
        ensure_master(ctx, fd);
        const TrainShape t = train_shape(fd);
        ctx->alloc(ctx->train_scratch, train_scratch_floats(t, (uint32_t)n) * 4);
        Stage st(ctx, INSTA_STAGE_TRAIN, 8 + 2 * (t.n_density + t.n_rgb) + extra_k);
        CK(launch_field_train(ctx->blas, tv, t, (const float*)fd.w32.p, coords, stride, (uint32_t)n, dl_dout, out4, grad,
                              (float*)ctx->train_scratch.p, ctx->stream, dl_dextra));
    });
}

int insta_train_set_math(insta_ctx* ctx, int math) {
    return guarded(ctx, [&] {
        if (math != INSTA_TRAIN_MATH_FP32 && math != INSTA_TRAIN_MATH_TF32 && math != INSTA_TRAIN_MATH_TCGEN05)
            fail(INSTA_ERR_INVALID_ARG, "unknown training math %d", math);
        ctx->train_tf32 = math == INSTA_TRAIN_MATH_TF32;
        ctx->train_tc = math == INSTA_TRAIN_MATH_TCGEN05;
        if (ctx->blas && cublasSetMathMode(ctx->blas, ctx->train_tf32 ? CUBLAS_TF32_TENSOR_OP_MATH : CUBLAS_DEFAULT_MATH) != CUBLAS_STATUS_SUCCESS)
            fail(INSTA_ERR_CUDA, "cublasSetMathMode failed");
    });
}

int insta_adam_step(insta_ctx* ctx, int avatar, const float* grad, const insta_adam_config* cfg) {
    return guarded(ctx, [&] {
        if (!grad || !cfg) fail(INSTA_ERR_INVALID_ARG, "null gradient or configuration");
        Avatar& a = ctx->avatar(avatar);
        Field& fd = a.field;
        if (!fd.ready) fail(INSTA_ERR_NOT_READY, "avatar %d has no field parameters", avatar);
        ensure_master(ctx, fd);
        if (!(cfg->ema_decay >= 0.f && cfg->ema_decay < 1.f)) fail(INSTA_ERR_INVALID_ARG, "ema_decay must be in [0, 1)");
        if (!(cfg->loss_scale >= 0.f) || isinf(cfg->loss_scale)) fail(INSTA_ERR_INVALID_ARG, "loss_scale must be finite and >= 0");
        const float loss_scale = cfg->loss_scale > 0.f ? cfg->loss_scale : 1.f;
        const uint64_t n_matrix = field_layout(fd.desc).table_off;
        if (fd.adam_step == 0) {
            ctx->alloc(fd.adam_m, fd.n_params * 4);
            ctx->alloc(fd.adam_v, fd.n_params * 4);
            ctx->alloc(fd.adam_steps, (fd.n_params - n_matrix) * 4);
            CK(cudaMemsetAsync(fd.adam_m.p, 0, fd.n_params * 4, ctx->stream));
            CK(cudaMemsetAsync(fd.adam_v.p, 0, fd.n_params * 4, ctx->stream));
            CK(cudaMemsetAsync(fd.adam_steps.p, 0, (fd.n_params - n_matrix) * 4, ctx->stream));
        }
        ctx->alloc(fd.w16, fd.n_params * 2);
        const uint32_t step = ++fd.adam_step;
        float* ema = nullptr;
        if (cfg->ema_decay > 0.f) {
            ctx->alloc(fd.ema, fd.n_params * 4);
            ema = (float*)fd.ema.p;
            ++fd.ema_step;
        } else {
            fd.ema_step = 0;   // a step without the Ema restarts its average
        }
        if (ema) ctx->alloc(fd.w16_train, fd.n_params * 2);
        {
            Stage st(ctx, INSTA_STAGE_TRAIN, 1);
            CK(launch_adam(fd.n_params, n_matrix, (float*)fd.w32.p, (float*)fd.adam_m.p, (float*)fd.adam_v.p, (uint32_t*)fd.adam_steps.p,
                           grad, loss_scale, cfg->learning_rate, cfg->beta1, cfg->beta2, cfg->epsilon, cfg->l2_reg, step, ema,
                           cfg->ema_decay, fd.ema_step, (__half*)fd.w16.p,
                           ema ? (__half*)fd.w16_train.p : nullptr, ctx->stream));
        }
        if (ema) {
            // the training weights' parameters and image: loaded like any parameters, then moved aside
            const insta_field_desc d0 = fd.desc;
            ctx->keep_master = true;
            const int rc0 = insta_params_load(ctx, avatar, &d0, (const uint16_t*)fd.w16_train.p, fd.n_params);
            ctx->keep_master = false;
            if (rc0 != INSTA_OK) fail(rc0, "%s", ctx->last_error.c_str());
            std::swap(fd.params, fd.train_params);
            std::swap(fd.image, fd.train_image);
            fd.train_view = fd.view;
            fd.train_valid = true;
        } else {
            fd.train_valid = false;
        }
        // the new FP16 parameters: the field's buffer and weight image (the master stays FP32)
        const insta_field_desc desc = fd.desc;
        ctx->keep_master = true;
        const int rc = insta_params_load(ctx, avatar, &desc, (const uint16_t*)fd.w16.p, fd.n_params);
        ctx->keep_master = false;
        if (rc != INSTA_OK) fail(rc, "%s", ctx->last_error.c_str());
    });
}

int insta_train_loss(insta_ctx* ctx, const insta_train_loss_desc* d) {
    return guarded(ctx, [&] {
        if (!d) fail(INSTA_ERR_INVALID_ARG, "null loss description");
        if (d->max_rays >= (1u << 26) || d->max_samples_compacted >= (1u << 28)) fail(INSTA_ERR_INVALID_ARG, "batch too large");
        if (d->n_rays == 0) fail(INSTA_ERR_INVALID_ARG, "n_rays must be positive");
        if (d->target_batch_size > d->max_samples_compacted) fail(INSTA_ERR_INVALID_ARG, "target_batch_size exceeds max_samples_compacted");
        if (d->stride < 11) fail(INSTA_ERR_INVALID_ARG, "stride too small");
        if (d->loss_type < 0 || d->loss_type > 6 || d->depth_loss_type < 0 || d->depth_loss_type > 6)
            fail(INSTA_ERR_INVALID_ARG, "unknown loss type");
        if (!d->numsteps_counter || !d->rays_counter) fail(INSTA_ERR_INVALID_ARG, "null counters");
        if (d->max_rays == 0) {
            if (d->target_batch_size > 0 && !(d->coords_out && d->dloss_doutput)) fail(INSTA_ERR_INVALID_ARG, "null output buffers");
        } else if (!d->rays || !d->target || !d->ray_indices || !d->numsteps || !d->coords || !d->network_output || !d->coords_out ||
                   !d->dloss_doutput) {
            fail(INSTA_ERR_INVALID_ARG, "null buffers");
        }
        if (((uintptr_t)d->network_output | (uintptr_t)d->dloss_doutput) & 15)
            fail(INSTA_ERR_INVALID_ARG, "network_output and dloss_doutput must be 16-byte aligned");
        if (d->error_map) {
            if (!d->image_xy || !d->image_index) fail(INSTA_ERR_INVALID_ARG, "the error map needs image_xy and image_index");
            if (d->error_map_res[0] < 2 || d->error_map_res[1] < 2 || (uint64_t)d->error_map_res[0] * d->error_map_res[1] > (1ull << 26))
                fail(INSTA_ERR_INVALID_ARG, "error_map_res must be at least 2 x 2 and at most 2^26 cells");
            if (d->error_map_images == 0) fail(INSTA_ERR_INVALID_ARG, "error_map_images must be positive");
            if ((uintptr_t)d->image_xy & 7) fail(INSTA_ERR_INVALID_ARG, "image_xy must be 8-byte aligned");
        }
        {
            ctx->alloc(ctx->loss_scratch, (size_t)std::max(d->max_rays, 1u) * 4);
            Stage st(ctx, INSTA_STAGE_TRAIN, (d->max_rays > 0 ? 2 : 0) + (d->target_batch_size > 0 ? 2 : 0));
            CK(launch_train_loss(*d, (uint32_t*)ctx->loss_scratch.p, ctx->stream));
        }
    });
}

int insta_training_pixels(insta_ctx* ctx, const insta_training_pixels_desc* d) {
    return guarded(ctx, [&] {
        if (!d) fail(INSTA_ERR_INVALID_ARG, "null description");
        if (d->n_rays == 0) return;
        if (d->n_images == 0) fail(INSTA_ERR_INVALID_ARG, "n_images must be positive");
        if (!d->out_image || !d->out_xy) fail(INSTA_ERR_INVALID_ARG, "null outputs");
        if (d->snap_to_pixel_centers && !d->resolution) fail(INSTA_ERR_INVALID_ARG, "snapping needs the image resolutions");
        const bool cdf = d->cdf_x_cond_y || d->cdf_y || d->cdf_img;
        if (cdf && !(d->cdf_x_cond_y && d->cdf_y && d->cdf_img)) fail(INSTA_ERR_INVALID_ARG, "give all three CDFs or none");
        if (cdf && (d->cdf_res[0] == 0 || d->cdf_res[1] == 0)) fail(INSTA_ERR_INVALID_ARG, "cdf_res must be positive");
        Stage st(ctx, INSTA_STAGE_TRAIN, 1);
        CK(launch_training_pixels(*d, ctx->stream));
    });
}

int insta_extra_dims_gradient(insta_ctx* ctx, const insta_extra_dims_gradient_desc* d) {
    return guarded(ctx, [&] {
        if (!d) fail(INSTA_ERR_INVALID_ARG, "null description");
        if (d->max_rays == 0 || d->n_extra_dims == 0) return;
        if (d->n_extra_dims > 256 || d->max_rays >= (1u << 26)) fail(INSTA_ERR_INVALID_ARG, "sizes out of range");
        if (!d->rays_counter || !d->ray_indices || !d->numsteps || !d->image_index || !d->dl_dextra || !d->extra_dims_gradient)
            fail(INSTA_ERR_INVALID_ARG, "null buffers");
        Stage st(ctx, INSTA_STAGE_TRAIN, 1);
        CK(launch_extra_dims_gradient(*d, ctx->stream));
    });
}

int insta_error_map_cdf(insta_ctx* ctx, const float* error_map, uint32_t n_images, uint32_t res_x, uint32_t res_y, float* cdf_x_cond_y,
                        float* cdf_y, float* cdf_img, float* pmf_img) {
    return guarded(ctx, [&] {
        if (n_images == 0 || res_x == 0 || res_y == 0) fail(INSTA_ERR_INVALID_ARG, "empty error map");
        if (n_images > 65535u) fail(INSTA_ERR_INVALID_ARG, "at most 65535 images");
        if (!error_map || !cdf_x_cond_y || !cdf_y || !cdf_img) fail(INSTA_ERR_INVALID_ARG, "null buffers");
        Stage st(ctx, INSTA_STAGE_TRAIN, 3);
        CK(launch_error_map_cdf(error_map, n_images, res_x, res_y, cdf_x_cond_y, cdf_y, cdf_img, pmf_img, ctx->stream));
    });
}

int insta_field_eval_static(insta_ctx* ctx, int avatar, const float* coords, uint32_t stride, int64_t n, float* out4) {
    return guarded(ctx, [&] {
        Avatar& a = ctx->avatar(avatar);
        if (!a.field.ready) fail(INSTA_ERR_NOT_READY, "avatar %d has no field parameters", avatar);
        if (n < 0 || (n > 0 && (!coords || !out4))) fail(INSTA_ERR_INVALID_ARG, "bad buffers");
        if (n > static_max_samples())
            fail(INSTA_ERR_INVALID_ARG, "insta_field_eval_static takes at most %lld samples per call, got %lld",
                 (long long)static_max_samples(), (long long)n);
        if (stride < 11 + a.field.desc.n_extra_dims) fail(INSTA_ERR_INVALID_ARG, "stride too small");
        if (n == 0) return;
        uint8_t* tiles = nullptr;
        uint2* out = nullptr;
        float4* out_f32 = nullptr;
        CK(static_scratch(ctx->device, &tiles, &out, &out_f32));
        const TilePlan& P = a.field.plan;
        const uint64_t n_tiles = ((uint64_t)n + 127) / 128;
        Stage st(ctx, INSTA_STAGE_FIELD, 3);
        CK(launch_encode_coords(a.field.view, coords, stride, n, tiles, P.tile_bytes, P.k_in, ctx->stream));
        MlpArgs m{};
        m.fv = a.field.view; m.plan = P; m.tiles = tiles; m.n_alive = nullptr; m.n_samples = n;
        m.out = out; m.out_f32 = out_f32; m.err = ctx->err_dev;
        CK(launch_mlp(m, (uint32_t)n_tiles, ctx->stream));
        CK(launch_unpack(out, out_f32, a.field.view.precision != 0, n, (float4*)out4, ctx->stream));
    });
}

int insta_render(insta_ctx* ctx, const insta_render_desc* req, float* out_rgba, float* out_depth) {
    return guarded(ctx, [&] { render_batch(ctx, req, 1, &out_rgba, &out_depth); });
}

int insta_render_async(insta_ctx* ctx, const insta_render_desc* req, float* out_rgba, float* out_depth) {
    return guarded(ctx, [&] { render_batch(ctx, req, 1, &out_rgba, &out_depth, true); });
}

int insta_render_batch(insta_ctx* ctx, const insta_render_desc* reqs, int n, float* const* out_rgba, float* const* out_depth) {
    return guarded(ctx, [&] {
        if (!reqs || !out_rgba || !out_depth) fail(INSTA_ERR_INVALID_ARG, "null request or output arrays");
        render_batch(ctx, reqs, n, out_rgba, out_depth);
    });
}

int insta_render_samples(insta_ctx* ctx, uint64_t* n_samples) {
    return guarded(ctx, [&] {
        if (!n_samples) fail(INSTA_ERR_INVALID_ARG, "null output");
        ctx->check_device();
        unsigned long long v = 0;
        CK(cudaMemcpy(&v, ctx->sample_counter, sizeof(v), cudaMemcpyDeviceToHost));
        *n_samples = v;
    });
}

int insta_tuning_set(insta_ctx* ctx, const insta_tuning* t) {
    return guarded(ctx, [&] {
        if (!t) fail(INSTA_ERR_INVALID_ARG, "null tuning");
        if (t->max_steps_per_round > kMaxSteps) fail(INSTA_ERR_INVALID_ARG, "max_steps_per_round must be 0..%u", kMaxSteps);
        if (t->sort_cell_bits && (t->sort_cell_bits < 12 || t->sort_cell_bits > 21 || t->sort_cell_bits % 3))
            fail(INSTA_ERR_INVALID_ARG, "sort_cell_bits must be 0 or one of 12, 15, 18, 21");
        if (t->mlp_ctas_per_sm > 4) fail(INSTA_ERR_INVALID_ARG, "mlp_ctas_per_sm must be 0..4");
        if (t->deform_blocks_per_sm > 64) fail(INSTA_ERR_INVALID_ARG, "deform_blocks_per_sm must be 0..64");
        if (t->bvh_top_nodes != 0 && t->bvh_top_nodes != 5 && t->bvh_top_nodes != 21)
            fail(INSTA_ERR_INVALID_ARG, "bvh_top_nodes must be 0, 5 or 21");
        if (t->fused_field_stage > 1) fail(INSTA_ERR_INVALID_ARG, "fused_field_stage must be 0 or 1");
        if (t->mlp_slots > 8) fail(INSTA_ERR_INVALID_ARG, "mlp_slots must be 0..8");
        ctx->tune = *t;
    });
}

int insta_tuning_get(insta_ctx* ctx, insta_tuning* t) {
    return guarded(ctx, [&] {
        if (!t) fail(INSTA_ERR_INVALID_ARG, "null output");
        *t = ctx->tune;
    });
}

int insta_autotune(insta_ctx* ctx, const insta_render_desc* reqs, int n, int repeats, insta_tuning* best, float* best_ms) {
    return guarded(ctx, [&] {
        if (!reqs || n <= 0 || (uint32_t)n > kMaxRequests) fail(INSTA_ERR_INVALID_ARG, "bad request list");
        if (repeats < 1 || repeats > 64) fail(INSTA_ERR_INVALID_ARG, "repeats must be 1..64");
        uint64_t px = 0;
        for (int i = 0; i < n; ++i) {
            check_request(reqs + i);
            px += (uint64_t)reqs[i].width * reqs[i].height;
        }
        ctx->alloc(ctx->tune_rgba, px * 16);
        ctx->alloc(ctx->tune_depth, px * 4);
        std::vector<float*> o_rgba((size_t)n), o_depth((size_t)n);
        {
            uint64_t off = 0;
            for (int i = 0; i < n; ++i) {
                o_rgba[(size_t)i] = (float*)ctx->tune_rgba.p + off * 4;
                o_depth[(size_t)i] = (float*)ctx->tune_depth.p + off;
                off += (uint64_t)reqs[i].width * reqs[i].height;
            }
        }
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        const bool timing = ctx->timing;
        ctx->timing = false;   // the timed path: the whole loop as one graph launch
        auto time_one = [&](const insta_tuning& t) {
            ctx->tune = t;
            render_batch(ctx, reqs, n, o_rgba.data(), o_depth.data());   // untimed: graph (re)built
            std::vector<float> ms((size_t)repeats);
            for (int k = 0; k < repeats; ++k) {
                CK(cudaEventRecord(e0, ctx->stream));
                render_batch(ctx, reqs, n, o_rgba.data(), o_depth.data());
                CK(cudaEventRecord(e1, ctx->stream));
                CK(cudaEventSynchronize(e1));
                CK(cudaEventElapsedTime(&ms[(size_t)k], e0, e1));
            }
            std::sort(ms.begin(), ms.end());
            return ms[ms.size() / 2];
        };
        insta_tuning cur = ctx->tune;
        float cur_ms = 0.f;
        try {
            cur_ms = time_one(cur);
            const std::vector<uint32_t> cands[7] = {{8, 16, 32, 64, 96, 128}, {15, 18, 21}, {1, 2, 3, 4}, {8, 12, 16, 24}, {0, 5, 21}, {0, 1},
                                                    {1, 7, 8}};
            for (int pass = 0; pass < 2; ++pass) {
                bool moved = false;
                for (int f = 0; f < 7; ++f) {
                    for (uint32_t v : cands[f]) {
                        insta_tuning t = cur;
                        uint32_t* field = f == 0 ? &t.max_steps_per_round : f == 1 ? &t.sort_cell_bits : f == 2 ? &t.mlp_ctas_per_sm
                                        : f == 3 ? &t.deform_blocks_per_sm : f == 4 ? &t.bvh_top_nodes : f == 5 ? &t.fused_field_stage
                                        : &t.mlp_slots;
                        if (*field == v) continue;
                        *field = v;
                        const float ms = time_one(t);
                        if (ms < cur_ms * 0.99f) { cur = t; cur_ms = ms; moved = true; }
                    }
                }
                if (!moved) break;
            }
        } catch (...) {
            ctx->timing = timing;
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            throw;
        }
        ctx->timing = timing;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        ctx->tune = cur;
        if (best) *best = cur;
        if (best_ms) *best_ms = cur_ms;
    });
}

int insta_stats_enable(insta_ctx* ctx, int stage_timing) {
    return guarded(ctx, [&] {
        ctx->collect_timings();
        ctx->timing = stage_timing != 0;
    });
}

int insta_stats_read(insta_ctx* ctx, insta_stats* out, int reset) {
    return guarded(ctx, [&] {
        if (!out) fail(INSTA_ERR_INVALID_ARG, "null output");
        ctx->collect_timings();
        if (ctx->loop_rounds_total) {
            // graph-run rounds: loop_round_kernels per round, plus the mid and end kernels per loop
            // iteration (the device total holds rounds in its low 40 bits, iterations above)
            unsigned long long total = 0;
            CK(cudaMemcpy(&total, ctx->loop_rounds_total, sizeof(total), cudaMemcpyDeviceToHost));
            const unsigned long long d = total - ctx->loop_rounds_seen;
            ctx->launches += (d & ((1ull << 40) - 1ull)) * ctx->loop_round_kernels + (d >> 40) * 2ull;
            ctx->loop_rounds_seen = total;
        }
        out->kernel_launches = ctx->launches;
        unsigned long long v = 0;
        CK(cudaMemcpy(&v, ctx->sample_counter, sizeof(v), cudaMemcpyDeviceToHost));
        out->last_render_samples = v;
        for (int k = 0; k < INSTA_STAGE_COUNT; ++k) {
            out->stage_ms[k] = (float)ctx->stage_ms[k];
            out->stage_calls[k] = ctx->stage_calls[k];
        }
        unsigned long long walk[8] = {};
        if (ctx->walk_stats) CK(cudaMemcpy(walk, ctx->walk_stats, sizeof(walk), cudaMemcpyDeviceToHost));
        out->walk_warps = walk[0];
        out->walk_inner_nodes = walk[1];
        out->walk_leaves = walk[2];
        out->walk_bound_tests = walk[3];
        out->walk_exact_tests = walk[4];
        if (reset) {
            ctx->launches = 0;
            for (int k = 0; k < INSTA_STAGE_COUNT; ++k) { ctx->stage_ms[k] = 0.0; ctx->stage_calls[k] = 0; }
            if (ctx->walk_stats) CK(cudaMemset(ctx->walk_stats, 0, 8 * sizeof(unsigned long long)));
        }
    });
}

int insta_march_debug(insta_ctx* ctx, const insta_render_desc* req, int max_out, float* out_t, float* out_dt, int32_t* out_n) {
    return guarded(ctx, [&] {
        check_request(req);
        if (max_out <= 0 || !out_t || !out_dt || !out_n) fail(INSTA_ERR_INVALID_ARG, "bad output buffers");
        Avatar& a = ctx->avatar(req->avatar);
        Frame& f = use_frame(ctx, a, req->frame);
        if (!f.has_occupancy) fail(INSTA_ERR_NOT_READY, "frame %d has no occupancy bitfield", req->frame);
        CK(launch_march_debug(render_view(a, *req), (const uint8_t*)f.bitfield.p, max_out, out_t, out_dt, out_n, ctx->stream));
    });
}

int insta_raycast(insta_ctx* ctx, const insta_render_desc* req, int color_normal, float* out_rgba, float* out_depth, int32_t* out_tri) {
    return guarded(ctx, [&] {
        check_request(req);
        if (!out_rgba || !out_depth) fail(INSTA_ERR_INVALID_ARG, "null output");
        Avatar& a = ctx->avatar(req->avatar);
        Frame& f = use_frame(ctx, a, req->frame);
        const size_t px = (size_t)req->width * req->height;
        // host outputs go through device staging (pixels without a hit keep their values)
        float* rgba = out_rgba;
        float* depth = out_depth;
        int32_t* tri = out_tri;
        const bool h_rgba = !is_device_ptr(out_rgba), h_depth = !is_device_ptr(out_depth), h_tri = out_tri && !is_device_ptr(out_tri);
        if (h_rgba) { rgba = (float*)ctx->alloc(ctx->out_rgba, px * 16); host_copy(rgba, out_rgba, px * 16, ctx->stream); }
        if (h_depth) { depth = (float*)ctx->alloc(ctx->out_depth, px * 4); host_copy(depth, out_depth, px * 4, ctx->stream); }
        if (h_tri) tri = (int32_t*)ctx->alloc(ctx->extra, px * 4);
        {
            Stage st(ctx, INSTA_STAGE_RAYCAST, 1);
            CK(launch_raycast(render_view(a, *req), f.view, a.center, color_normal, rgba, depth, tri, ctx->err_dev, ctx->stream));
        }
        if (h_rgba) host_copy(out_rgba, rgba, px * 16, ctx->stream);
        if (h_depth) host_copy(out_depth, depth, px * 4, ctx->stream);
        if (h_tri) host_copy(out_tri, tri, px * 4, ctx->stream);
        if (h_rgba || h_depth || h_tri) ctx->check_device();
    });
}

int insta_nearest_debug(insta_ctx* ctx, int avatar, int frame, const float* pts, int64_t n, int32_t* out_idx) {
    return guarded(ctx, [&] {
        if (n < 0 || (n > 0 && (!pts || !out_idx))) fail(INSTA_ERR_INVALID_ARG, "bad buffers");
        Avatar& a = ctx->avatar(avatar);
        Frame& f = use_frame(ctx, a, frame);
        CK(launch_nearest_debug(f.view, pts, n, out_idx, ctx->err_dev, ctx->stream));
    });
}

}  // extern "C"

// ------------------------------------------------------------------------------- serving
// A request loop over one context: render requests (each with its own tracked-mesh frame) are
// admitted into request slots as slots and the pixel budget free up, and their rays join the
// running wavefront at the next round -- requests that arrive while others are on the GPU overlap
// with them on the device.  A slot is released as soon as its last ray has composited.
namespace {

using Clock = std::chrono::steady_clock;
constexpr int kServerFrameBase = 1 << 30;   // frame ids the server uses for request frames

struct ServerReq {
    uint64_t ticket = 0;
    insta_render_desc desc{};
    std::vector<float> extra, verts;
    float* out_rgba = nullptr;
    float* out_depth = nullptr;
    bool host_out = false;
    int state = INSTA_REQ_QUEUED;
    int slot = -1;
    bool cancel = false;
    bool started = false;   // its rays are in the wavefront
    bool copying = false;   // rays done; its host outputs are being copied back (copy stream)
    std::string error;
    Clock::time_point t_submit, t_start, t_done;
};

}  // namespace

struct insta_server {
    insta_ctx* ctx = nullptr;
    insta_server_config cfg{};
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<ServerReq>> queue;
    std::unordered_map<uint64_t, std::shared_ptr<ServerReq>> tickets;
    bool stop = false, failed = false;
    std::string fail_msg;
    uint64_t next_ticket = 1;
    uint64_t completed = 0, rounds = 0;
    // worker-owned
    std::vector<std::shared_ptr<ServerReq>> slot_req;
    std::vector<ReqView> views;
    std::vector<DevBuf> slot_rgba, slot_depth;
    DevBuf slot_extra;
    WaveRun run;
    const Field* layout = nullptr;
    uint64_t inflight_px = 0;
    int inflight = 0;
    // admitted requests' frames are built on a second stream while the current round runs;
    // their rays start at the next round, after `ev_ready`
    cudaStream_t side = nullptr;
    cudaEvent_t ev_ready = nullptr;
    std::vector<std::shared_ptr<ServerReq>> ready;
    // output copies back to the host on the context's copy stream, after the rounds (ev_rounds)
    cudaEvent_t ev_rounds = nullptr;
    std::vector<cudaEvent_t> slot_copied;

    void finish(const std::shared_ptr<ServerReq>& r, int state, const std::string& err = std::string()) {
        std::lock_guard<std::mutex> lk(mu);
        r->state = state;
        r->error = err;
        r->t_done = Clock::now();
        ++completed;
        cv_done.notify_all();
    }

    // Upload the admitted requests' frames and build their LBVHs (one launch per avatar, a CTA per
    // frame) and occupancy on the side stream, and fill their slots.  A request that cannot run
    // is finished as failed without disturbing the others.
    void build(std::vector<std::shared_ptr<ServerReq>>& batch) {
        std::map<int, std::vector<std::shared_ptr<ServerReq>>> by_avatar;
        for (auto& r : batch) {
            try {
                Avatar& a = ctx->avatar(r->desc.avatar);
                if (!a.field.ready) fail(INSTA_ERR_NOT_READY, "avatar %d has no field parameters", r->desc.avatar);
                if (!layout) {
                    layout = &a.field;
                    run.setup(ctx, a.field, cfg.max_inflight, cfg.max_inflight_pixels, true,
                              cfg.round_samples ? cfg.round_samples : kMaxRoundSamples);
                } else if (!same_field_layout(*layout, a.field)) {
                    fail(INSTA_ERR_UNSUPPORTED, "the server's requests must share one field layout");
                }
                if (r->verts.empty()) {
                    Frame& f = get_frame(a, r->desc.frame);
                    if (!f.has_occupancy) fail(INSTA_ERR_NOT_READY, "frame %d has no occupancy bitfield", r->desc.frame);
                }
                by_avatar[r->desc.avatar].push_back(r);
            } catch (const Failure& e) {
                release(r);
                finish(r, INSTA_REQ_FAILED, e.what());
            }
        }
        bool any = false;
        for (auto& kv : by_avatar) {
            Avatar& a = ctx->avatar(kv.first);
            std::vector<FrameView> fviews;
            std::vector<const float*> dverts;
            for (auto& r : kv.second) {
                if (r->verts.empty()) continue;
                Frame& f = prepare_frame(ctx, a, kServerFrameBase + r->slot, r->verts.data(), side);
                ctx->alloc(f.bitfield, (size_t)8 * GRID3 / 8);
                fviews.push_back(f.view);
                dverts.push_back((const float*)f.verts.p);
            }
            if (!fviews.empty()) {
                const int n = (int)fviews.size();
                ctx->alloc(ctx->bvh_scratch, (size_t)n * bvh_scratch_bytes(a.F));
                ctx->alloc(ctx->frame_jobs, frame_batch_table_bytes(n));
                CK(launch_frames_batch(n, a.F, fviews.data(), dverts.data(), (const int32_t*)a.faces.p, (const uint32_t*)a.mask.p,
                                       (const float*)a.canon_area.p, ctx->bvh_scratch.p, ctx->frame_jobs.p, side));
                ctx->launches += 3;
            }
            for (auto& r : kv.second) {
                int frame = r->desc.frame;
                if (!r->verts.empty()) {
                    frame = kServerFrameBase + r->slot;
                    Frame& f = get_frame(a, frame);
                    CK(launch_occupancy(f.view, cfg.occupancy_radius, (uint8_t*)f.bitfield.p, ctx->err_dev, side));
                    ctx->launches += 1;
                    f.has_occupancy = true;
                }
                Frame& f = get_frame(a, frame);
                insta_render_desc d = r->desc;
                d.frame = frame;
                ReqView v = request_view(ctx, d, a, f);
                const size_t px = (size_t)d.width * d.height;
                const uint32_t s = (uint32_t)r->slot;
                if (r->host_out) {
                    v.out_rgba = (float*)ctx->alloc(slot_rgba[s], px * 16);
                    v.out_depth = (float*)ctx->alloc(slot_depth[s], px * 4);
                } else {
                    v.out_rgba = r->out_rgba;
                    v.out_depth = r->out_depth;
                }
                const uint32_t n_extra = layout->view.n_extra;
                v.extra = nullptr;
                if (n_extra) {
                    std::vector<float> e(n_extra, 0.f);
                    if (!r->extra.empty()) std::memcpy(e.data(), r->extra.data(), n_extra * 4);
                    float* dst = (float*)slot_extra.p + (size_t)s * n_extra;
                    // pageable source: staged before the call returns
                    CK(cudaMemcpyAsync(dst, e.data(), n_extra * 4, cudaMemcpyHostToDevice, side));
                    v.extra = dst;
                }
                views[s] = v;
                ready.push_back(r);
                any = true;
            }
        }
        if (any) CK(cudaEventRecord(ev_ready, side));
    }

    // Start the rays of the requests built in the previous iteration (after their build).
    void start_ready() {
        if (ready.empty()) return;
        CK(cudaStreamWaitEvent(ctx->stream, ev_ready, 0));
        std::vector<uint32_t> slots, tiles;
        for (auto& r : ready) {
            const uint32_t s = (uint32_t)r->slot;
            CK(cudaMemsetAsync(run.W.req_alive + s, 0, 4, ctx->stream));
            slots.push_back(s);
            tiles.push_back(views[s].tiles);
        }
        run.upload_table(views.data());
        run.start(slots.data(), tiles.data(), (uint32_t)slots.size(), false);
        std::lock_guard<std::mutex> lk(mu);
        for (auto& r : ready) {
            r->started = true;
            r->state = INSTA_REQ_RUNNING;
            r->t_start = Clock::now();
        }
        ready.clear();
    }

    void release(const std::shared_ptr<ServerReq>& r) {
        if (r->slot < 0) return;
        slot_req[(size_t)r->slot] = nullptr;
        inflight_px -= (uint64_t)r->desc.width * r->desc.height;
        --inflight;
        r->slot = -1;
    }

    // After a round: requests whose rays have all composited are done.  Host outputs are copied
    // back on the copy stream (page-locked host buffers let the copies overlap the next rounds);
    // such a request keeps its slot until its copy has landed (poll_copies).
    void collect() {
        bool any_copy = false;
        for (size_t s = 0; s < slot_req.size(); ++s) {
            auto r = slot_req[s];
            if (!r || !r->started || r->copying || r->state != INSTA_REQ_RUNNING || ctx->host_alive[s] != 0) continue;
            if (r->host_out && !r->cancel) {
                if (!any_copy) {
                    CK(cudaEventRecord(ev_rounds, ctx->stream));
                    CK(cudaStreamWaitEvent(ctx->copy, ev_rounds, 0));
                    any_copy = true;
                }
                const size_t px = (size_t)r->desc.width * r->desc.height;
                CK(cudaMemcpyAsync(r->out_rgba, slot_rgba[s].p, px * 16, cudaMemcpyDeviceToHost, ctx->copy));
                CK(cudaMemcpyAsync(r->out_depth, slot_depth[s].p, px * 4, cudaMemcpyDeviceToHost, ctx->copy));
                CK(cudaEventRecord(slot_copied[s], ctx->copy));
                r->copying = true;
                continue;
            }
            release(r);
            finish(r, r->cancel ? INSTA_REQ_CANCELLED : INSTA_REQ_DONE);
        }
        poll_copies(false);
    }

    // Requests whose output copies have landed are done; `wait_one` blocks for the oldest copy
    // when nothing else is left to run.
    void poll_copies(bool wait_one) {
        for (size_t s = 0; s < slot_req.size(); ++s) {
            auto r = slot_req[s];
            if (!r || !r->copying) continue;
            cudaError_t q = wait_one ? cudaEventSynchronize(slot_copied[s]) : cudaEventQuery(slot_copied[s]);
            if (q == cudaErrorNotReady) continue;
            CK(q);
            wait_one = false;
            r->copying = false;
            release(r);
            finish(r, INSTA_REQ_DONE);
        }
    }

    bool any_copying() const {
        for (auto& r : slot_req)
            if (r && r->copying) return true;
        return false;
    }

    void loop() {
        cudaSetDevice(ctx->device);
        try {
            CK(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&ev_ready, cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&ev_rounds, cudaEventDisableTiming));
            ensure_copy_stream(ctx);
            slot_copied.resize(cfg.max_inflight);
            for (auto& e : slot_copied) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            ctx->alloc(slot_extra, (size_t)cfg.max_inflight * 64 * 4);
            for (;;) {
                std::vector<std::shared_ptr<ServerReq>> batch;
                {
                    std::unique_lock<std::mutex> lk(mu);
                    cv_work.wait(lk, [&] { return stop || inflight > 0 || !queue.empty(); });
                    if (stop && inflight == 0) break;
                    while (!stop && !queue.empty() && inflight < (int)cfg.max_inflight) {
                        auto r = queue.front();
                        const uint64_t px = (uint64_t)r->desc.width * r->desc.height;
                        if (r->cancel) {
                            queue.pop_front();
                            r->state = INSTA_REQ_CANCELLED;
                            r->t_done = Clock::now();
                            ++completed;
                            cv_done.notify_all();
                            continue;
                        }
                        if (inflight > 0 && inflight_px + px > cfg.max_inflight_pixels) break;   // wait for pixels to free up
                        if (ctx->budget && inflight > 0 && ctx->used + px * 20 + (8u << 20) > ctx->budget) break;   // memory
                        queue.pop_front();
                        size_t s = 0;
                        while (slot_req[s]) ++s;
                        slot_req[s] = r;
                        r->slot = (int)s;
                        inflight_px += px;
                        ++inflight;
                        batch.push_back(r);
                    }
                }
                const bool had_ready = !ready.empty();
                start_ready();
                if (!batch.empty()) build(batch);
                if (inflight == 0) continue;
                if (run.n_alive == 0 && !had_ready) {
                    // nothing to march: either frames still building (start them next) or only
                    // output copies in flight (wait for the oldest)
                    if (ready.empty() && batch.empty() && any_copying()) poll_copies(true);
                    continue;
                }
                if (ctx->timing) {
                    run.round();
                    ++rounds;
                } else {
                    // the rounds up to the next admission point as one CUDA-graph launch (a
                    // conditional while node stopping early when no ray is alive), then one host
                    // read of the alive counts
                    const uint32_t k = cfg.rounds_per_launch ? cfg.rounds_per_launch : 2u;
                    run.device_rounds(k);
                    run.n_alive = run.read_alive();
                    rounds += k;
                }
                collect();
            }
        } catch (const std::exception& e) {
            std::lock_guard<std::mutex> lk(mu);
            failed = true;
            fail_msg = e.what();
            for (auto& kv : tickets)
                if (kv.second->state == INSTA_REQ_QUEUED || kv.second->state == INSTA_REQ_RUNNING) {
                    kv.second->state = INSTA_REQ_FAILED;
                    kv.second->error = fail_msg;
                    kv.second->t_done = Clock::now();
                }
            queue.clear();
            cv_done.notify_all();
        }
    }
};

extern "C" {

int insta_server_create(insta_ctx* ctx, const insta_server_config* cfg, insta_server** out) {
    return guarded(ctx, [&] {
        if (!cfg || !out) fail(INSTA_ERR_INVALID_ARG, "null config or output");
        if (cfg->max_inflight < 1 || cfg->max_inflight > 256) fail(INSTA_ERR_INVALID_ARG, "max_inflight must be 1..256");
        if (cfg->max_inflight_pixels < 1 || cfg->max_inflight_pixels > kMaxBatchPixels)
            fail(INSTA_ERR_INVALID_ARG, "max_inflight_pixels must be 1..2^25");
        if (!(cfg->occupancy_radius > 0.0)) fail(INSTA_ERR_INVALID_ARG, "occupancy_radius must be positive");
        if (cfg->rounds_per_launch % 2 || cfg->rounds_per_launch > 64) fail(INSTA_ERR_INVALID_ARG, "rounds_per_launch must be even, 0..64");
        if (cfg->round_samples && (cfg->round_samples < (1ull << 16) || cfg->round_samples > kMaxRoundSamples))
            fail(INSTA_ERR_INVALID_ARG, "round_samples must be 0 or 2^16..2^25");
        auto s = std::make_unique<insta_server>();
        s->ctx = ctx;
        s->cfg = *cfg;
        s->slot_req.resize(cfg->max_inflight);
        s->views.resize(cfg->max_inflight);
        s->slot_rgba.resize(cfg->max_inflight);
        s->slot_depth.resize(cfg->max_inflight);
        insta_server* raw = s.get();
        s->worker = std::thread([raw] { raw->loop(); });
        *out = s.release();
    });
}

int insta_server_destroy(insta_server* s) {
    if (!s) return INSTA_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (auto& r : s->queue) { r->state = INSTA_REQ_CANCELLED; r->t_done = Clock::now(); }
        s->queue.clear();
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();   // in-flight requests finish first
    if (s->side) { cudaStreamSynchronize(s->side); cudaStreamDestroy(s->side); }
    if (s->ev_ready) cudaEventDestroy(s->ev_ready);
    if (s->ctx->copy) cudaStreamSynchronize(s->ctx->copy);
    if (s->ev_rounds) cudaEventDestroy(s->ev_rounds);
    for (auto& e : s->slot_copied) cudaEventDestroy(e);
    for (auto& b : s->slot_rgba) s->ctx->release(b);
    for (auto& b : s->slot_depth) s->ctx->release(b);
    s->ctx->release(s->slot_extra);
    delete s;
    return INSTA_OK;
}

int insta_submit(insta_server* s, const insta_render_desc* req, const float* frame_verts, float* out_rgba, float* out_depth,
                 uint64_t* ticket) {
    if (!s || !req || !out_rgba || !out_depth || !ticket) return INSTA_ERR_INVALID_ARG;
    try {
        check_request(req);
    } catch (const Failure& e) {
        return e.code;
    }
    if ((uint64_t)req->width * req->height > s->cfg.max_inflight_pixels) return INSTA_ERR_INVALID_ARG;
    auto r = std::make_shared<ServerReq>();
    r->desc = *req;
    r->desc.extra_dims = nullptr;
    // avatars are not added or removed while the server runs, so reading them here is safe
    auto it = s->ctx->avatars.find(req->avatar);
    if (it == s->ctx->avatars.end()) return INSTA_ERR_NOT_READY;
    const Avatar& a = *it->second;
    if (req->extra_dims && a.field.ready)
        r->extra.assign(req->extra_dims, req->extra_dims + a.field.desc.n_extra_dims);
    if (frame_verts) r->verts.assign(frame_verts, frame_verts + (size_t)a.V * 3);
    r->out_rgba = out_rgba;
    r->out_depth = out_depth;
    r->host_out = !(is_device_ptr(out_rgba) && is_device_ptr(out_depth));
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->failed || s->stop) return INSTA_ERR_DEVICE;
        r->ticket = s->next_ticket++;
        s->tickets[r->ticket] = r;
        s->queue.push_back(r);
        *ticket = r->ticket;
    }
    s->cv_work.notify_one();
    return INSTA_OK;
}

int insta_poll(insta_server* s, uint64_t ticket, int* state, double* latency_ms) {
    if (!s || !state) return INSTA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return INSTA_ERR_INVALID_ARG;
    *state = it->second->state;
    if (latency_ms) {
        const auto& r = *it->second;
        *latency_ms = r.state >= INSTA_REQ_DONE ? std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count() : -1.0;
    }
    return INSTA_OK;
}

int insta_wait(insta_server* s, uint64_t ticket, int timeout_ms, int* state) {
    if (!s || !state) return INSTA_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return INSTA_ERR_INVALID_ARG;
    auto r = it->second;
    auto done = [&] { return r->state >= INSTA_REQ_DONE; };
    if (timeout_ms < 0) s->cv_done.wait(lk, done);
    else s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done);
    *state = r->state;
    return INSTA_OK;
}

int insta_cancel(insta_server* s, uint64_t ticket) {
    if (!s) return INSTA_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->tickets.find(ticket);
        if (it == s->tickets.end()) return INSTA_ERR_INVALID_ARG;
        it->second->cancel = true;   // queued: dropped at admission; running: finishes, outputs not delivered
    }
    s->cv_work.notify_one();
    return INSTA_OK;
}

int insta_server_release(insta_server* s, uint64_t ticket) {
    if (!s) return INSTA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return INSTA_ERR_INVALID_ARG;
    if (it->second->state < INSTA_REQ_DONE) return INSTA_ERR_NOT_READY;
    s->tickets.erase(it);
    return INSTA_OK;
}

const char* insta_server_error(insta_server* s, uint64_t ticket) {
    if (!s) return "null server";
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it != s->tickets.end() && !it->second->error.empty()) return it->second->error.c_str();
    return s->failed ? s->fail_msg.c_str() : "";
}

}  // extern "C"
