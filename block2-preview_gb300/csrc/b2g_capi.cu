// C ABI entry points (declared in include/b2g.h): context, H_eff plan
// creation/upload, H_eff*psi in the FP64, FP32 and TF32x3 (tensor-core)
// forms for one or several roots, diag(H_eff), timing and the FP64 probe.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "b2g_internal.h"

namespace b2g {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
    set_error(msg);
    return code;
}

static std::atomic<uint64_t> g_launches{0};
static thread_local int g_capturing = 0;
static thread_local uint64_t g_captured = 0;

void note_launch(uint64_t n) {
    if (g_capturing)
        g_captured += n;
    else
        g_launches.fetch_add(n, std::memory_order_relaxed);
}
void capture_begin() { g_capturing = 1, g_captured = 0; }
uint64_t capture_end() {
    g_capturing = 0;
    return g_captured;
}

template <typename T> static int upload(const std::vector<T> &v, T **dst, cudaStream_t s) {
    *dst = nullptr;
    if (v.empty())
        return B2G_OK;
    if (cudaMalloc((void **)dst, sizeof(T) * v.size()) != cudaSuccess) {
        *dst = nullptr;
        return fail(B2G_ERR_NOMEM, "cudaMalloc failed for plan table");
    }
    B2G_CUDA_TRY(cudaMemcpyAsync(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
    return B2G_OK;
}

static void free_plan(DevicePlan &p) {
    cudaFree(p.works), cudaFree(p.contribs), cudaFree(p.regions);
    cudaFree(p.t1), cudaFree(p.t2), cudaFree(p.lists);
    cudaFree(p.t2multi), cudaFree(p.g0tile), cudaFree(p.g0col);
    cudaFree(p.g1tile), cudaFree(p.g1stage), cudaFree(p.g1task), cudaFree(p.g1aimg);
    cudaFree(p.g1red), cudaFree(p.g1cover), cudaFree(p.region_cb);
    cudaFree(p.diag_task), cudaFree(p.diag_tlist), cudaFree(p.diag_item);
    p = DevicePlan();
}

// drop every captured apply (their buffers are about to move, or the H_eff goes)
static void clear_graphs(b2g_heff *h) {
    for (auto &g : h->graphs)
        if (g.exec)
            cudaGraphExecDestroy(g.exec);
    h->graphs.clear();
}

// per-root buffers (work matrices, split-K partials, float psi) for nroots roots
static int ensure_roots(b2g_heff *h, int nroots) {
    if (nroots <= h->cap_roots)
        return B2G_OK;
    B2G_CUDA_TRY(cudaStreamSynchronize(h->ctx->stream));
    clear_graphs(h);
    cudaFree(h->work), cudaFree(h->simt_part), cudaFree(h->psi32);
    h->work = nullptr, h->simt_part = nullptr, h->psi32 = nullptr;
    h->cap_roots = 0;
    const size_t R = (size_t)nroots;
    if ((h->work_size && cudaMalloc(&h->work, sizeof(double) * h->work_size * R) != cudaSuccess) ||
        (h->simt_part_size &&
         cudaMalloc(&h->simt_part, sizeof(double) * h->simt_part_size * R) != cudaSuccess) ||
        (h->psi_size && cudaMalloc(&h->psi32, sizeof(float) * h->psi_size * R) != cudaSuccess)) {
        cudaFree(h->work), cudaFree(h->simt_part), cudaFree(h->psi32);
        h->work = nullptr, h->simt_part = nullptr, h->psi32 = nullptr;
        return fail(B2G_ERR_NOMEM, "cudaMalloc failed for the per-root work buffers of " +
                                       std::to_string(nroots) + " roots");
    }
    h->cap_roots = nroots;
    return B2G_OK;
}

// buffers of the image-fed tensor-core GEMM1 (TF32x3 form only, made on its
// first use): A images once, W images and partial tiles per root
static int ensure_g1(b2g_heff *h, int nroots) {
    const DevicePlan &p = h->plan;
    if (h->g1_aimg == nullptr && p.g1_abytes) {
        if (cudaMalloc(&h->g1_aimg, p.g1_abytes) != cudaSuccess) {
            h->g1_aimg = nullptr;
            return fail(B2G_ERR_NOMEM, "cudaMalloc failed for the GEMM1 operator images");
        }
        B2G_CUDA_TRY(launch_g1_build_a(p, h->ops32, h->g1_aimg, h->ctx->stream));
    }
    if (nroots <= h->g1_roots)
        return B2G_OK;
    B2G_CUDA_TRY(cudaStreamSynchronize(h->ctx->stream));
    clear_graphs(h);
    cudaFree(h->g1_wimg), cudaFree(h->g1_part), cudaFree(h->g0_psi);
    h->g1_wimg = nullptr, h->g1_part = nullptr, h->g0_psi = nullptr, h->g1_roots = 0;
    const size_t R = (size_t)nroots;
    if ((p.g1_wbytes && cudaMalloc(&h->g1_wimg, p.g1_wbytes * R) != cudaSuccess) ||
        (p.g1_part && cudaMalloc(&h->g1_part, sizeof(float) * p.g1_part * R) != cudaSuccess) ||
        (p.g0_psi_floats && cudaMalloc(&h->g0_psi, sizeof(float) * p.g0_psi_floats * R) != cudaSuccess)) {
        cudaFree(h->g1_wimg), cudaFree(h->g1_part), cudaFree(h->g0_psi);
        h->g1_wimg = nullptr, h->g1_part = nullptr, h->g0_psi = nullptr;
        return fail(B2G_ERR_NOMEM, "cudaMalloc failed for the GEMM1 work images of " +
                                       std::to_string(nroots) + " roots");
    }
    // the padding of the W images (rows past m0 in the last K slab, columns past
    // n0) is never written by GEMM0 and must read as zero
    if (p.g1_wbytes)
        B2G_CUDA_TRY(cudaMemsetAsync(h->g1_wimg, 0, p.g1_wbytes * R, h->ctx->stream));
    h->g1_roots = nroots;
    return B2G_OK;
}

// replace the device plan of h by hp: drops the captured graphs and every
// plan-shaped buffer (images, partials), which the next apply rebuilds
static int install_plan(b2g_heff *h, const HostPlan &hp) {
    cudaStream_t s = h->ctx->stream;
    B2G_CUDA_TRY(cudaStreamSynchronize(s));
    clear_graphs(h);
    free_plan(h->plan);
    cudaFree(h->g1_aimg), cudaFree(h->g1_wimg), cudaFree(h->g1_part), cudaFree(h->g0_psi);
    h->g1_aimg = nullptr, h->g1_wimg = nullptr, h->g1_part = nullptr, h->g0_psi = nullptr;
    h->g1_roots = 0;
    DevicePlan &p = h->plan;
    int rc;
    if ((rc = upload(hp.works, &p.works, s)) || (rc = upload(hp.contribs, &p.contribs, s)) ||
        (rc = upload(hp.regions, &p.regions, s)) || (rc = upload(hp.t1, &p.t1, s)) ||
        (rc = upload(hp.t2, &p.t2, s)) || (rc = upload(hp.lists, &p.lists, s)) ||
        (rc = upload(hp.t2multi, &p.t2multi, s)) ||
        (rc = upload(hp.g0tile, &p.g0tile, s)) || (rc = upload(hp.g0col, &p.g0col, s)) ||
        (rc = upload(hp.g1tile, &p.g1tile, s)) ||
        (rc = upload(hp.g1stage, &p.g1stage, s)) || (rc = upload(hp.g1task, &p.g1task, s)) ||
        (rc = upload(hp.g1aimg, &p.g1aimg, s)) ||
        (rc = upload(hp.g1red, &p.g1red, s)) || (rc = upload(hp.g1cover, &p.g1cover, s)) ||
        (rc = upload(hp.g0psi, &p.g0psi, s)) || (rc = upload(hp.region_cb, &p.region_cb, s)) ||
        (rc = upload(hp.diag_task, &p.diag_task, s)) || (rc = upload(hp.diag_tlist, &p.diag_tlist, s)) ||
        (rc = upload(hp.diag_item, &p.diag_item, s)))
        return rc;
    p.n_g1task = (int64_t)hp.g1task.size(), p.n_g1aimg = (int64_t)hp.g1aimg.size();
    p.n_g1red = (int64_t)hp.g1red.size(), p.n_g0tile = (int64_t)hp.g0tile.size();
    p.n_g0psi = (int64_t)hp.g0psi.size(), p.g0_psi_floats = hp.g0_psi_floats;
    p.n_g0wide = hp.g0_wide;
    p.n_diag_task = (int64_t)hp.diag_task.size();
    p.g1_abytes = hp.g1_abytes, p.g1_wbytes = hp.g1_wbytes, p.g1_part = hp.g1_part;
    p.n_t2multi = (int64_t)hp.t2multi.size();
    p.n_works = (int64_t)hp.works.size(), p.n_contribs = (int64_t)hp.contribs.size();
    p.n_regions = (int64_t)hp.regions.size(), p.n_t1 = (int64_t)hp.t1.size();
    p.n_t2 = (int64_t)hp.t2.size(), p.n_lists = (int64_t)hp.lists.size();
    h->params = hp.params;
    if (cudaStreamSynchronize(s) != cudaSuccess)
        return fail(B2G_ERR_CUDA, "plan upload failed");
    return B2G_OK;
}

} // namespace b2g

using namespace b2g;

extern "C" {

int b2g_version(void) { return 1; }

const char *b2g_last_error(void) { return g_last_error.c_str(); }

int b2g_context_create(int device, b2g_context **out) {
    if (out == nullptr)
        return fail(B2G_ERR_ARG, "b2g_context_create: null output");
    *out = nullptr;
    int n = 0;
    B2G_CUDA_TRY(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n)
        return fail(B2G_ERR_ARG, "b2g_context_create: no CUDA device " + std::to_string(device));
    B2G_CUDA_TRY(cudaSetDevice(device));
    cudaDeviceProp prop;
    B2G_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    if (prop.major * 10 + prop.minor < 100)
        return fail(B2G_ERR_UNSUPPORTED, std::string("b2g: device ") + prop.name +
                                             " is not a Blackwell (sm_10x) GPU");
    b2g_context *c = new b2g_context();
    c->device = device;
    c->n_sm = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return fail(B2G_ERR_CUDA, "cudaStreamCreate failed");
    }
    *out = c;
    return B2G_OK;
}

int b2g_context_destroy(b2g_context *ctx) {
    if (ctx == nullptr)
        return B2G_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
    if (ctx->host_buf != nullptr)
        cudaFreeHost(ctx->host_buf);
    delete ctx;
    return B2G_OK;
}

int b2g_host_buffer(b2g_context *ctx, uint64_t bytes, void **out) {
    if (ctx == nullptr || out == nullptr)
        return fail(B2G_ERR_ARG, "b2g_host_buffer: null argument");
    *out = nullptr;
    B2G_CUDA_TRY(cudaSetDevice(ctx->device));
    if (bytes > ctx->host_buf_bytes) {
        // copies out of the old buffer may still be in flight
        B2G_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        if (ctx->host_buf != nullptr)
            cudaFreeHost(ctx->host_buf);
        ctx->host_buf = nullptr, ctx->host_buf_bytes = 0;
        // grow by a quarter beyond the request, so a slowly growing sweep does
        // not reallocate at every site
        const uint64_t want = bytes + bytes / 4;
        if (cudaHostAlloc(&ctx->host_buf, want, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            ctx->host_buf = nullptr;
            return fail(B2G_ERR_NOMEM, "cudaHostAlloc failed for the pinned staging buffer");
        }
        ctx->host_buf_bytes = want;
    }
    *out = ctx->host_buf;
    return B2G_OK;
}

void *b2g_context_stream(b2g_context *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int b2g_context_synchronize(b2g_context *ctx) {
    if (ctx == nullptr)
        return fail(B2G_ERR_ARG, "null context");
    B2G_CUDA_TRY(cudaSetDevice(ctx->device));
    B2G_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return B2G_OK;
}

int b2g_heff_create(b2g_context *ctx, const b2g_pair_seq *seq, const double *ops,
                    uint64_t ops_size, int ops_on_device, uint64_t psi_size, uint64_t sigma_size,
                    b2g_heff **out) {
    const bool deferred = ops_on_device == B2G_OPS_DEFERRED;
    if (ctx == nullptr || seq == nullptr || out == nullptr || (ops == nullptr && ops_size != 0 && !deferred))
        return fail(B2G_ERR_ARG, "b2g_heff_create: null argument");
    *out = nullptr;
    B2G_CUDA_TRY(cudaSetDevice(ctx->device));
    HostPlan hp;
    int rc = build_plan(seq, ops_size, psi_size, sigma_size, hp);
    if (rc != B2G_OK)
        return rc;
    b2g_heff *h = new b2g_heff();
    h->ctx = ctx;
    h->ops_size = ops_size, h->psi_size = psi_size, h->sigma_size = sigma_size;
    h->work_size = hp.work_size;
    auto bail = [&](int code) {
        free_plan(h->plan);
        cudaFree(h->ops), cudaFree(h->work), cudaFree(h->err);
        cudaFree(h->simt_part), cudaFree(h->psi32);
        cudaFree(h->g1_aimg), cudaFree(h->g1_wimg), cudaFree(h->g1_part), cudaFree(h->g0_psi);
        delete h;
        return code;
    };
    cudaStream_t s = ctx->stream;
    if (ops_size) {
        if (cudaMalloc(&h->ops, sizeof(double) * ops_size) != cudaSuccess) {
            h->ops = nullptr;
            return bail(fail(B2G_ERR_NOMEM, "cudaMalloc failed for the operator blob"));
        }
        if (!deferred && cudaMemcpyAsync(h->ops, ops, sizeof(double) * ops_size,
                                         ops_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                         s) != cudaSuccess)
            return bail(fail(B2G_ERR_CUDA, "operator blob upload failed"));
    }
    h->simt_part_size = (uint64_t)4 * 256 * hp.t2_part_tiles;
    if ((rc = ensure_roots(h, 1)) != B2G_OK)
        return bail(rc);
    if (cudaMalloc(&h->err, sizeof(int)) != cudaSuccess) {
        h->err = nullptr;
        return bail(fail(B2G_ERR_NOMEM, "cudaMalloc failed for the error flag"));
    }
    if (cudaMemsetAsync(h->err, 0, sizeof(int), s) != cudaSuccess)
        return bail(fail(B2G_ERR_CUDA, "error flag reset failed"));
    if ((rc = install_plan(h, hp)) != B2G_OK)
        return bail(rc);
    const DevicePlan &p = h->plan;
    b2g_heff_stats &st = h->stats;
    st.n_pairs = seq->n_pairs;
    st.n_work = p.n_works;
    st.n_regions = p.n_regions;
    st.n_tiles = p.n_t2;
    st.mnk = hp.mnk;
    st.mnk_executed = hp.mnk_exec;
    st.ops_bytes = sizeof(double) * ops_size;
    st.work_bytes = sizeof(double) * hp.work_size;
    st.plan_bytes = sizeof(WorkDesc) * hp.works.size() + sizeof(Contrib) * hp.contribs.size() +
                    sizeof(Region) * hp.regions.size() + sizeof(Task1) * hp.t1.size() +
                    sizeof(Task2) * hp.t2.size() + sizeof(int32_t) * hp.lists.size() +
                    sizeof(G1Tile) * hp.g1tile.size() + sizeof(G1Stage) * hp.g1stage.size() +
                    sizeof(G1Task) * hp.g1task.size() + sizeof(G1AImg) * hp.g1aimg.size() +
                    sizeof(G1WImg) * hp.g1wimg.size() + sizeof(G1Red) * hp.g1red.size();
    st.psi_size = psi_size, st.sigma_size = sigma_size;
    *out = h;
    return B2G_OK;
}

int b2g_heff_status(b2g_heff *h) {
    if (h == nullptr)
        return fail(B2G_ERR_ARG, "b2g_heff_status: null handle");
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    B2G_CUDA_TRY(cudaStreamSynchronize(h->ctx->stream));
    int e = 0;
    B2G_CUDA_TRY(cudaMemcpy(&e, h->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e != 0)
        return fail(B2G_ERR_STATE, "b2g: a tensor-core kernel gave up a bounded wait; its sigma is incomplete");
    return B2G_OK;
}

int b2g_heff_destroy(b2g_heff *h) {
    if (h == nullptr)
        return B2G_OK;
    cudaSetDevice(h->ctx->device);
    cudaStreamSynchronize(h->ctx->stream);
    clear_graphs(h);
    free_adjoint(h);
    free_plan(h->plan);
    cudaFree(h->ops), cudaFree(h->ops32), cudaFree(h->psi32), cudaFree(h->work);
    cudaFree(h->simt_part);
    cudaFree(h->g1_aimg), cudaFree(h->g1_wimg), cudaFree(h->g1_part), cudaFree(h->g0_psi);
    cudaFree(h->psi_stage), cudaFree(h->sigma_stage), cudaFree(h->err);
    for (auto &e : h->ev)
        if (e)
            cudaEventDestroy(e);
    delete h;
    return B2G_OK;
}

int b2g_heff_diag(b2g_heff *h, double *diag) {
    if (h == nullptr || (h->sigma_size && diag == nullptr))
        return fail(B2G_ERR_ARG, "b2g_heff_diag: null argument");
    if (h->psi_size != h->sigma_size)
        return fail(B2G_ERR_UNSUPPORTED, "b2g_heff_diag: bra and ket spaces differ");
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    cudaStream_t s = h->ctx->stream;
    B2G_CUDA_TRY(cudaMemsetAsync(diag, 0, sizeof(double) * h->sigma_size, s));
    B2G_CUDA_TRY(launch_diag(h->plan, h->ops, diag, s));
    return B2G_OK;
}

int b2g_heff_diag_host(b2g_heff *h, double *diag) {
    if (h == nullptr || (h->sigma_size && diag == nullptr))
        return fail(B2G_ERR_ARG, "b2g_heff_diag_host: null argument");
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    double *d = nullptr;
    if (h->sigma_size && cudaMalloc(&d, sizeof(double) * h->sigma_size) != cudaSuccess)
        return fail(B2G_ERR_NOMEM, "b2g_heff_diag_host: cudaMalloc failed");
    int rc = b2g_heff_diag(h, d);
    if (rc == B2G_OK && h->sigma_size) {
        cudaError_t e = cudaMemcpyAsync(diag, d, sizeof(double) * h->sigma_size, cudaMemcpyDeviceToHost,
                                        h->ctx->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(h->ctx->stream);
        if (e != cudaSuccess)
            rc = fail(B2G_ERR_CUDA, std::string("b2g_heff_diag_host: ") + cudaGetErrorString(e));
    }
    cudaFree(d);
    return rc;
}

int b2g_heff_set_timing(b2g_heff *h, int enable) {
    if (h == nullptr)
        return fail(B2G_ERR_ARG, "b2g_heff_set_timing: null handle");
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    if (enable && h->ev[0] == nullptr)
        for (auto &e : h->ev)
            B2G_CUDA_TRY(cudaEventCreate(&e));
    h->timing = enable != 0;
    return B2G_OK;
}

int b2g_heff_last_timing(b2g_heff *h, float *ms) {
    if (h == nullptr || ms == nullptr)
        return fail(B2G_ERR_ARG, "b2g_heff_last_timing: null argument");
    if (!h->timing)
        return fail(B2G_ERR_STATE, "b2g_heff_last_timing: timing not enabled");
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    B2G_CUDA_TRY(cudaEventSynchronize(h->ev[2]));
    B2G_CUDA_TRY(cudaEventElapsedTime(&ms[0], h->ev[0], h->ev[1]));
    B2G_CUDA_TRY(cudaEventElapsedTime(&ms[1], h->ev[1], h->ev[2]));
    return B2G_OK;
}

int b2g_probe_peak(b2g_context *ctx, int form, double *tflops) {
    if (ctx == nullptr || tflops == nullptr)
        return fail(B2G_ERR_ARG, "b2g_probe_peak: null argument");
    B2G_CUDA_TRY(cudaSetDevice(ctx->device));
    if (form == B2G_FP64) {
        B2G_CUDA_TRY(probe_fp64_peak(ctx->stream, ctx->n_sm, tflops));
        return B2G_OK;
    }
    if (form == B2G_PROBE_FP64_MMA) {
        B2G_CUDA_TRY(probe_fp64_mma_peak(ctx->stream, ctx->n_sm, tflops));
        return B2G_OK;
    }
    return fail(B2G_ERR_UNSUPPORTED, "b2g_probe_peak: form not available");
}

int b2g_heff_stats_get(const b2g_heff *h, b2g_heff_stats *out) {
    if (h == nullptr || out == nullptr)
        return fail(B2G_ERR_ARG, "b2g_heff_stats_get: null argument");
    *out = h->stats;
    return B2G_OK;
}

int b2g_launch_count(uint64_t *out) {
    if (out == nullptr)
        return fail(B2G_ERR_ARG, "b2g_launch_count: null argument");
    *out = g_launches.load(std::memory_order_relaxed);
    return B2G_OK;
}

int b2g_plan_stats(const b2g_pair_seq *seq, uint64_t ops_size, uint64_t psi_size,
                   uint64_t sigma_size, b2g_heff_stats *out) {
    if (seq == nullptr || out == nullptr)
        return fail(B2G_ERR_ARG, "b2g_plan_stats: null argument");
    HostPlan hp;
    int rc = build_plan(seq, ops_size, psi_size, sigma_size, hp);
    if (rc != B2G_OK)
        return rc;
    b2g_heff_stats st{};
    st.n_pairs = seq->n_pairs;
    st.n_work = (int64_t)hp.works.size();
    st.n_regions = (int64_t)hp.regions.size();
    st.n_tiles = (int64_t)hp.t2.size();
    st.mnk = hp.mnk;
    st.mnk_executed = hp.mnk_exec;
    st.ops_bytes = sizeof(double) * ops_size;
    st.work_bytes = sizeof(double) * hp.work_size;
    st.plan_bytes = sizeof(WorkDesc) * hp.works.size() + sizeof(Contrib) * hp.contribs.size() +
                    sizeof(Region) * hp.regions.size() + sizeof(Task1) * hp.t1.size() +
                    sizeof(Task2) * hp.t2.size() + sizeof(int32_t) * hp.lists.size();
    st.psi_size = psi_size, st.sigma_size = sigma_size;
    *out = st;
    return B2G_OK;
}

} // extern "C"

namespace b2g {

// buffers and one-time conversions an apply needs (allocations, syncs: never
// inside a stream capture)
static int apply_prepare(b2g_heff *h, int nroots, int form) {
    int rc = ensure_roots(h, nroots);
    if (rc != B2G_OK)
        return rc;
    if (form == B2G_FP32 || form == B2G_TF32X3) {
        if (h->ops32 == nullptr && h->ops_size) {
            if (cudaMalloc(&h->ops32, sizeof(float) * h->ops_size) != cudaSuccess) {
                h->ops32 = nullptr;
                return fail(B2G_ERR_NOMEM, "cudaMalloc failed for the float operator copy");
            }
            B2G_CUDA_TRY(launch_to_float(h->ops, h->ops32, h->ops_size, h->ctx->stream));
        }
        if (form == B2G_TF32X3 && (rc = ensure_g1(h, nroots)) != B2G_OK)
            return rc;
    }
    return B2G_OK;
}

// the kernel launches of one apply (stream-ordered only: capturable)
static int apply_launches(b2g_heff *h, const double *psi, double *sigma, int nroots, double scale,
                          int form) {
    cudaStream_t s = h->ctx->stream;
    RootStrides rs;
    rs.nroots = nroots, rs.psi = h->psi_size, rs.sigma = h->sigma_size;
    if (form == B2G_FP64) {
        rs.work = h->work_size, rs.part = h->simt_part_size;
        if (h->timing)
            B2G_CUDA_TRY(cudaEventRecord(h->ev[0], s));
        B2G_CUDA_TRY(launch_simt_phase1<double>(h->plan, h->ops, psi, h->work, rs, s));
        if (h->timing)
            B2G_CUDA_TRY(cudaEventRecord(h->ev[1], s));
        B2G_CUDA_TRY(launch_simt_phase2<double>(h->plan, h->ops, h->work, sigma, (double *)h->simt_part,
                                                scale, rs, s));
        if (h->timing)
            B2G_CUDA_TRY(cudaEventRecord(h->ev[2], s));
        return B2G_OK;
    }
    float *w32 = (float *)h->work;
    rs.work = 2 * h->work_size;  // floats per root in a buffer sized in doubles
    if (h->timing)
        B2G_CUDA_TRY(cudaEventRecord(h->ev[0], s));
    if (form == B2G_TF32X3) {
        // psi enters as a packed FP32 copy of its sub-blocks (made by launch_g0)
        rs.wimg = h->plan.g1_wbytes, rs.part = h->plan.g1_part;
        B2G_CUDA_TRY(launch_g0(h->plan, h->g1_aimg, psi, h->g0_psi, h->g1_wimg, h->err, rs, s));
    } else {
        // psi rounded once (FP64 conversions run on the narrow FP64 pipe of GB300)
        B2G_CUDA_TRY(launch_to_float(psi, h->psi32, h->psi_size * (uint64_t)nroots, s));
        B2G_CUDA_TRY(launch_simt_phase1<float>(h->plan, h->ops32, h->psi32, w32, rs, s));
    }
    if (h->timing)
        B2G_CUDA_TRY(cudaEventRecord(h->ev[1], s));
    if (form == B2G_TF32X3) {
        B2G_CUDA_TRY(launch_g1(h->plan, h->g1_aimg, h->g1_wimg, h->g1_part, sigma, scale, h->err, rs, s));
    } else {
        rs.part = 2 * h->simt_part_size;
        B2G_CUDA_TRY(launch_simt_phase2<float>(h->plan, h->ops32, w32, sigma, (float *)h->simt_part,
                                               scale, rs, s));
    }
    if (h->timing)
        B2G_CUDA_TRY(cudaEventRecord(h->ev[2], s));
    return B2G_OK;
}

// apply through the graph cache: first use of an argument set runs eagerly,
// the second captures and replays, later ones replay (LRU of kMaxApplyGraphs)
static int apply_graphed(b2g_heff *h, const double *psi, double *sigma, int nroots, double scale,
                         int form) {
    cudaStream_t s = h->ctx->stream;
    ApplyGraph *g = nullptr;
    for (auto &e : h->graphs)
        if (e.psi == psi && e.sigma == sigma && e.nroots == nroots && e.form == form &&
            memcmp(&e.scale, &scale, sizeof scale) == 0) {
            g = &e;
            break;
        }
    if (g == nullptr) {
        if (h->graphs.size() >= kMaxApplyGraphs) {
            size_t v = 0;
            for (size_t i = 1; i < h->graphs.size(); i++)
                if (h->graphs[i].last < h->graphs[v].last)
                    v = i;
            if (h->graphs[v].exec)
                cudaGraphExecDestroy(h->graphs[v].exec);
            h->graphs.erase(h->graphs.begin() + (ptrdiff_t)v);
        }
        ApplyGraph e;
        e.psi = psi, e.sigma = sigma, e.nroots = nroots, e.form = form, e.scale = scale;
        e.last = ++h->graph_tick;
        h->graphs.push_back(e);
        return apply_launches(h, psi, sigma, nroots, scale, form);
    }
    g->last = ++h->graph_tick;
    if (g->state == 1) {
        B2G_CUDA_TRY(cudaGraphLaunch(g->exec, s));
        note_launch(g->n_kernels);
        return B2G_OK;
    }
    if (g->state < 0)
        return apply_launches(h, psi, sigma, nroots, scale, form);
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        g->state = -1;
        return apply_launches(h, psi, sigma, nroots, scale, form);
    }
    capture_begin();
    const int rc = apply_launches(h, psi, sigma, nroots, scale, form);
    g->n_kernels = capture_end();
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s, &graph);
    if (rc != B2G_OK) {
        if (graph)
            cudaGraphDestroy(graph);
        return rc;
    }
    cudaError_t ei = cudaErrorUnknown;
    if (ec == cudaSuccess && graph != nullptr)
        ei = cudaGraphInstantiate(&g->exec, graph, 0);
    if (graph)
        cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        cudaGetLastError();
        g->exec = nullptr;
        g->state = -1;
        return apply_launches(h, psi, sigma, nroots, scale, form);
    }
    g->state = 1;
    B2G_CUDA_TRY(cudaGraphLaunch(g->exec, s));
    note_launch(g->n_kernels);
    return B2G_OK;
}

} // namespace b2g

extern "C" {

int b2g_heff_apply_batch(b2g_heff *h, const double *psi, double *sigma, int nroots, double scale,
                         int form) {
    if (h == nullptr || nroots < 1 || (h->psi_size && psi == nullptr) ||
        (h->sigma_size && sigma == nullptr))
        return fail(B2G_ERR_ARG, "b2g_heff_apply: null argument or nroots < 1");
    if (nroots > 65535)
        return fail(B2G_ERR_ARG, "b2g_heff_apply: too many roots");
    if (form != B2G_FP64 && form != B2G_FP32 && form != B2G_TF32X3)
        return fail(B2G_ERR_UNSUPPORTED, "b2g_heff_apply: unknown form " + std::to_string(form));
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    int rc = apply_prepare(h, nroots, form);
    if (rc != B2G_OK)
        return rc;
    if (h->graphs_on && !h->timing)
        return apply_graphed(h, psi, sigma, nroots, scale, form);
    return apply_launches(h, psi, sigma, nroots, scale, form);
}

// Autotuner of the tensor-core tile shapes.  The candidates come from the
// block-size histogram of the installed plan: narrower GEMM1 tiles only when
// some sigma rectangles are wider than 128 columns, narrower GEMM0 tiles only
// when some right operators are shared by more than 128 psi rows, and two
// split-K chunk lengths; each candidate plan is installed and timed (CUDA
// events, L2 flushed between applies) and the fastest is kept.
int b2g_heff_autotune(b2g_heff *h, const b2g_pair_seq *seq, int form, b2g_tune_result *res) {
    if (h == nullptr || seq == nullptr || res == nullptr)
        return fail(B2G_ERR_ARG, "b2g_heff_autotune: null argument");
    if (form != B2G_TF32X3)
        return fail(B2G_ERR_UNSUPPORTED, "b2g_heff_autotune: only the TF32x3 form has tile shapes");
    if (seq->n_pairs != h->stats.n_pairs)
        return fail(B2G_ERR_ARG, "b2g_heff_autotune: not the pair sequence of this H_eff");
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    cudaStream_t s = h->ctx->stream;
    *res = b2g_tune_result{};
    HostPlan hp;
    int rc = build_plan(seq, h->ops_size, h->psi_size, h->sigma_size, hp, PlanParams());
    if (rc != B2G_OK)
        return rc;
    if (hp.mnk != h->stats.mnk)
        return fail(B2G_ERR_ARG, "b2g_heff_autotune: not the pair sequence of this H_eff");
    // histogram: GEMM1 stage work in tiles wider than 128 columns, GEMM0 tiles
    // with more than 128 stacked rows
    double w1 = 0, w1_wide = 0;
    for (const G1Task &k : hp.g1task) {
        const G1Tile &tl = hp.g1tile[k.tile];
        w1 += (double)k.n_stages * tl.n;
        if (tl.n > 128)
            w1_wide += (double)k.n_stages * tl.n;
    }
    int64_t g0_wide = 0;
    for (const G0Tile &t : hp.g0tile)
        g0_wide += t.ncol > 128;
    res->g1_wide_frac = w1 > 0 ? w1_wide / w1 : 0.0;
    res->g0_wide_frac = hp.g0tile.empty() ? 0.0 : (double)g0_wide / (double)hp.g0tile.size();
    std::vector<PlanParams> cand;
    for (int c1 : {256, 128})
        for (int c0 : {256, 128})
            for (int ch : {kTcMaxChunkStages, kG1ChunkLimit, kTcMaxChunkStages / 2}) {
                if (c1 == 128 && w1_wide == 0)
                    continue;
                if (c0 == 128 && g0_wide == 0)
                    continue;
                PlanParams pp;
                pp.g1_tile_cols = c1, pp.g0_tile_cols = c0, pp.g1_chunk = ch;
                cand.push_back(pp);
            }
    // scratch: psi, sigma, and an L2 flush buffer larger than L2
    const size_t kFlush = (size_t)256 << 20;
    double *x = nullptr, *y = nullptr;
    unsigned char *flush = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
        cudaFree(x), cudaFree(y), cudaFree(flush);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    if (cudaMalloc(&x, sizeof(double) * std::max<uint64_t>(1, h->psi_size)) ||
        cudaMalloc(&y, sizeof(double) * std::max<uint64_t>(1, h->sigma_size)) ||
        cudaMalloc(&flush, kFlush) || cudaEventCreate(&e0) || cudaEventCreate(&e1)) {
        cleanup();
        return fail(B2G_ERR_NOMEM, "b2g_heff_autotune: scratch allocation failed");
    }
    const bool timing = h->timing;
    h->timing = false;
    int best = -1;
    float best_ms = 0.f;
    for (size_t i = 0; i < cand.size() && rc == B2G_OK; i++) {
        HostPlan cp;
        if ((rc = build_plan(seq, h->ops_size, h->psi_size, h->sigma_size, cp, cand[i])) != B2G_OK ||
            (rc = install_plan(h, cp)) != B2G_OK || (rc = apply_prepare(h, 1, form)) != B2G_OK)
            break;
        if (cudaMemsetAsync(x, 0x3F, sizeof(double) * h->psi_size, s) != cudaSuccess) {
            rc = fail(B2G_ERR_CUDA, "b2g_heff_autotune: scratch fill failed");
            break;
        }
        std::vector<float> ms;
        for (int rep = 0; rep < 7 && rc == B2G_OK; rep++) {
            cudaMemsetAsync(flush, rep, kFlush, s);
            cudaMemsetAsync(y, 0, sizeof(double) * h->sigma_size, s);
            cudaEventRecord(e0, s);
            rc = apply_launches(h, x, y, 1, 1.0, form);
            cudaEventRecord(e1, s);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                rc = fail(B2G_ERR_CUDA, "b2g_heff_autotune: timed apply failed");
                break;
            }
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            if (rep >= 2)
                ms.push_back(t);
        }
        if (rc != B2G_OK)
            break;
        std::sort(ms.begin(), ms.end());
        const float med = ms[ms.size() / 2];
        if (i < 12) {
            res->ms[i] = med;
            res->g0_tile_cols[i] = cand[i].g0_tile_cols;
            res->g1_tile_cols[i] = cand[i].g1_tile_cols;
            res->g1_chunk[i] = cand[i].g1_chunk;
        }
        if (best < 0 || med < best_ms)
            best = (int)i, best_ms = med;
    }
    res->n_candidates = (int32_t)std::min<size_t>(cand.size(), 12);
    res->best = best;
    if (rc == B2G_OK && best >= 0 && best + 1 != (int)cand.size()) {
        HostPlan bp;
        if ((rc = build_plan(seq, h->ops_size, h->psi_size, h->sigma_size, bp, cand[best])) == B2G_OK)
            rc = install_plan(h, bp);
    }
    h->timing = timing;
    if (rc == B2G_OK && b2g_heff_status(h) != B2G_OK)
        rc = B2G_ERR_STATE;
    cleanup();
    return rc;
}

int b2g_heff_set_params(b2g_heff *h, const b2g_pair_seq *seq, const int32_t *params) {
    if (h == nullptr || seq == nullptr || params == nullptr)
        return fail(B2G_ERR_ARG, "b2g_heff_set_params: null argument");
    if (seq->n_pairs != h->stats.n_pairs)
        return fail(B2G_ERR_ARG, "b2g_heff_set_params: not the pair sequence of this H_eff");
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    PlanParams pp;
    pp.g0_tile_cols = params[0], pp.g1_tile_cols = params[1], pp.g1_chunk = params[2];
    HostPlan hp;
    int rc = build_plan(seq, h->ops_size, h->psi_size, h->sigma_size, hp, pp);
    if (rc != B2G_OK)
        return rc;
    if (hp.mnk != h->stats.mnk)
        return fail(B2G_ERR_ARG, "b2g_heff_set_params: not the pair sequence of this H_eff");
    return install_plan(h, hp);
}

int b2g_heff_get_params(const b2g_heff *h, int32_t *params) {
    if (h == nullptr || params == nullptr)
        return fail(B2G_ERR_ARG, "b2g_heff_get_params: null argument");
    params[0] = h->params.g0_tile_cols, params[1] = h->params.g1_tile_cols;
    params[2] = h->params.g1_chunk;
    return B2G_OK;
}

int b2g_heff_set_graphs(b2g_heff *h, int enable) {
    if (h == nullptr)
        return fail(B2G_ERR_ARG, "b2g_heff_set_graphs: null handle");
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    if (!enable) {
        B2G_CUDA_TRY(cudaStreamSynchronize(h->ctx->stream));
        clear_graphs(h);
    }
    h->graphs_on = enable != 0;
    return B2G_OK;
}

int b2g_heff_graph_count(const b2g_heff *h) {
    if (h == nullptr)
        return -1;
    int n = 0;
    for (const auto &g : h->graphs)
        n += g.state == 1;
    return n;
}

int b2g_heff_apply(b2g_heff *h, const double *psi, double *sigma, double scale, int form) {
    return b2g_heff_apply_batch(h, psi, sigma, 1, scale, form);
}

int b2g_heff_apply_host(b2g_heff *h, const double *psi, double *sigma, double scale, int form) {
    if (h == nullptr || (h->psi_size && psi == nullptr) || (h->sigma_size && sigma == nullptr))
        return fail(B2G_ERR_ARG, "b2g_heff_apply_host: null argument");
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    cudaStream_t s = h->ctx->stream;
    if (h->psi_stage == nullptr && h->psi_size &&
        cudaMalloc(&h->psi_stage, sizeof(double) * h->psi_size) != cudaSuccess) {
        h->psi_stage = nullptr;
        return fail(B2G_ERR_NOMEM, "cudaMalloc failed for psi staging");
    }
    if (h->sigma_stage == nullptr && h->sigma_size &&
        cudaMalloc(&h->sigma_stage, sizeof(double) * h->sigma_size) != cudaSuccess) {
        h->sigma_stage = nullptr;
        return fail(B2G_ERR_NOMEM, "cudaMalloc failed for sigma staging");
    }
    B2G_CUDA_TRY(cudaMemcpyAsync(h->psi_stage, psi, sizeof(double) * h->psi_size,
                                 cudaMemcpyHostToDevice, s));
    B2G_CUDA_TRY(cudaMemcpyAsync(h->sigma_stage, sigma, sizeof(double) * h->sigma_size,
                                 cudaMemcpyHostToDevice, s));
    int rc = b2g_heff_apply(h, h->psi_stage, h->sigma_stage, scale, form);
    if (rc != B2G_OK)
        return rc;
    B2G_CUDA_TRY(cudaMemcpyAsync(sigma, h->sigma_stage, sizeof(double) * h->sigma_size,
                                 cudaMemcpyDeviceToHost, s));
    if (form == B2G_TF32X3)
        return b2g_heff_status(h);
    B2G_CUDA_TRY(cudaStreamSynchronize(s));
    return B2G_OK;
}

} // extern "C"
