// Quad4.update_KC0 (pyfe3d/quad4.pyx:1204-1313) on HOST buffers: the
// caller's coordinates, offsets, properties and COO arrays live in host
// memory (pinned for full overlap), as for the reference's own numpy arrays.
//
// The elements are streamed through the GPU in chunks on four streams:
// upload (offsets, property ids and the current values of the chunk's COO
// slots, which update_KC0 accumulates into), compute (the device KC0 kernel
// on the chunk), download of the values and, on a second stream, of the
// rows and columns.  Three staging sets let
// the upload of chunk c+1 and the download of chunk c-1 run while chunk c
// is computed, so the transfer time, not the sum of the three phases, sets
// the pace.  Requires the reference's contiguous layout init_k[e] =
// init_k[0] + 576 e (checked on the host; other layouts get FE3D_ERR_ARG
// and go through the device entry point with whole-array copies).
#include <mutex>

#include "common.cuh"

extern "C" int fe3d_quad4_kc0(int64_t E, const int64_t *cdof, const int64_t *init_k, const double *x, int64_t nx,
                              const double *xmat, int xmat_stride, const double *R, const double *m,
                              const double *xe, const double *area, const double *props, int64_t nprops,
                              const int32_t *pid, int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk,
                              int values_only, int *err, void *stream);

namespace fe3d {
namespace {

constexpr int kSets = 3;
constexpr int64_t kSlots = 576;

// Device staging kept between calls (grown on demand, one device at a time).
struct Staging {
    int dev = -1;
    size_t bytes = 0;
    unsigned char *base = nullptr;
};
Staging g_stage;
std::mutex g_mu;

unsigned char *staging(size_t bytes) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    if (g_stage.base && (g_stage.dev != dev || g_stage.bytes < bytes)) {
        cudaFree(g_stage.base);
        g_stage.base = nullptr;
        g_stage.bytes = 0;
    }
    if (!g_stage.base) {
        if (cudaMalloc((void **)&g_stage.base, bytes) != cudaSuccess) {
            g_stage.base = nullptr;
            return nullptr;
        }
        g_stage.dev = dev;
        g_stage.bytes = bytes;
    }
    return g_stage.base;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

__global__ void iota_kernel(int64_t n, int64_t step, int64_t *out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = step * i;
}

struct Streams {
    cudaStream_t s[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t up[kSets] = {}, done[kSets] = {}, down[kSets] = {}, down2[kSets] = {}, ev = nullptr;
    ~Streams() {
        for (int i = 0; i < kSets; i++) {
            if (up[i]) cudaEventDestroy(up[i]);
            if (done[i]) cudaEventDestroy(done[i]);
            if (down[i]) cudaEventDestroy(down[i]);
            if (down2[i]) cudaEventDestroy(down2[i]);
        }
        if (ev) cudaEventDestroy(ev);
        for (auto &q : s)
            if (q) cudaStreamDestroy(q);
    }
    bool init() {
        for (auto &q : s)
            if (cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking) != cudaSuccess) return false;
        for (int i = 0; i < kSets; i++)
            if (cudaEventCreateWithFlags(&up[i], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&down[i], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&down2[i], cudaEventDisableTiming) != cudaSuccess)
                return false;
        return cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
    }
};

}  // namespace
}  // namespace fe3d

using namespace fe3d;

extern "C" int fe3d_quad4_kc0_host(int64_t E, const int64_t *cdof, const int64_t *init_k, const double *x,
                                   int64_t nx, const double *props, int64_t nprops, const int32_t *pid,
                                   int64_t *Kr, int64_t *Kc, double *Kv, int64_t nk, int values_only,
                                   int64_t chunk, int *err_host, void *stream) {
    if (E < 0 || nx < 0 || nprops <= 0) return FE3D_ERR_ARG;
    if (E == 0) return FE3D_OK;
    if (!cdof || !init_k || !x || !props || !Kv || (!values_only && (!Kr || !Kc))) return FE3D_ERR_ARG;
    if (!pid && nprops < E) return FE3D_ERR_ARG;
    // the contiguous layout of the reference (Quad4Data offsets 576 apart)
    const int64_t k0 = init_k[0];
    for (int64_t e = 1; e < E; e++)
        if (init_k[e] != k0 + kSlots * e) return FE3D_ERR_ARG;
    if (k0 < 0 || k0 + kSlots * E > nk) return FE3D_ERR_BOUNDS;
    if (chunk <= 0) chunk = 65536;
    if (chunk > E) chunk = E;

    std::lock_guard<std::mutex> lock(g_mu);
    // staging: shared x, properties, iota offsets, error word; per set
    // cdof, pid and the chunk's Kr, Kc, Kv
    const size_t b_x = align256(sizeof(double) * (size_t)(nx > 0 ? nx : 1));
    const int64_t np_dev = pid ? nprops : chunk;  // without pid: record e per element, streamed
    const size_t b_p = align256(sizeof(double) * FE3D_SHELL_PROP_STRIDE * (size_t)np_dev);
    const size_t b_iota = align256(sizeof(int64_t) * (size_t)chunk);
    const size_t b_err = 256;
    const size_t b_cdof = align256(sizeof(int64_t) * 4 * (size_t)chunk);
    const size_t b_pid = align256(sizeof(int32_t) * (size_t)chunk);
    const size_t b_props_set = pid ? 0 : b_p;
    const size_t b_k = align256(sizeof(double) * kSlots * (size_t)chunk);
    const size_t per_set = b_cdof + b_pid + b_props_set + 3 * b_k;
    unsigned char *base = staging(b_x + (pid ? b_p : 0) + b_iota + b_err + kSets * per_set);
    if (!base) return FE3D_ERR_NOMEM;
    double *d_x = (double *)base;
    double *d_props = (double *)(base + b_x);
    unsigned char *q = base + b_x + (pid ? b_p : 0);
    int64_t *d_iota = (int64_t *)q;
    int *d_err = (int *)(q + b_iota);
    unsigned char *sets = q + b_iota + b_err;

    Streams S;
    if (!S.init()) return FE3D_ERR_CUDA;
    // values and indices come back on two streams (two copy queues)
    cudaStream_t up = S.s[0], comp = S.s[1], down = S.s[2], down2 = S.s[3];
    // ordered after the caller's earlier work
    FE3D_CUDA(cudaEventRecord(S.ev, as_stream(stream)));
    FE3D_CUDA(cudaStreamWaitEvent(up, S.ev, 0));
    FE3D_CUDA(cudaMemcpyAsync(d_x, x, sizeof(double) * nx, cudaMemcpyHostToDevice, up));
    if (pid)
        FE3D_CUDA(cudaMemcpyAsync(d_props, props, sizeof(double) * FE3D_SHELL_PROP_STRIDE * nprops,
                                  cudaMemcpyHostToDevice, up));
    FE3D_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), up));
    iota_kernel<<<(unsigned)((chunk + 255) / 256), 256, 0, up>>>(chunk, kSlots, d_iota);
    FE3D_CHECK_LAUNCH();
    int rc = FE3D_OK;
    // chunk sizes ramp up from chunk / 8, doubling: the first download starts
    // early and every chunk's upload and kernel take less time than the
    // previous chunk's download (the link, not the kernel, sets the pace)
    int64_t e0 = 0, want = chunk >= 4096 ? chunk / 8 : chunk;
    for (int64_t c = 0; e0 < E && rc == FE3D_OK; c++) {
        const int si = (int)(c % kSets);
        unsigned char *st = sets + si * per_set;
        int64_t *d_cdof = (int64_t *)st;
        int32_t *d_pid = (int32_t *)(st + b_cdof);
        double *d_pset = (double *)(st + b_cdof + b_pid);
        int64_t *d_kr = (int64_t *)(st + b_cdof + b_pid + b_props_set);
        int64_t *d_kc = (int64_t *)(st + b_cdof + b_pid + b_props_set + b_k);
        double *d_kv = (double *)(st + b_cdof + b_pid + b_props_set + 2 * b_k);
        const int64_t n = (E - e0 < want) ? E - e0 : want;
        const int64_t s0 = k0 + kSlots * e0, ns = kSlots * n;
        // upload (after the download that last used this set)
        if (c >= kSets) {
            FE3D_CUDA(cudaStreamWaitEvent(up, S.down[si], 0));
            FE3D_CUDA(cudaStreamWaitEvent(up, S.down2[si], 0));
        }
        FE3D_CUDA(cudaMemcpyAsync(d_cdof, cdof + 4 * e0, sizeof(int64_t) * 4 * n, cudaMemcpyHostToDevice, up));
        if (pid)
            FE3D_CUDA(cudaMemcpyAsync(d_pid, pid + e0, sizeof(int32_t) * n, cudaMemcpyHostToDevice, up));
        else
            FE3D_CUDA(cudaMemcpyAsync(d_pset, props + FE3D_SHELL_PROP_STRIDE * e0,
                                      sizeof(double) * FE3D_SHELL_PROP_STRIDE * n, cudaMemcpyHostToDevice, up));
        FE3D_CUDA(cudaMemcpyAsync(d_kv, Kv + s0, sizeof(double) * ns, cudaMemcpyHostToDevice, up));
        FE3D_CUDA(cudaEventRecord(S.up[si], up));
        // compute
        FE3D_CUDA(cudaStreamWaitEvent(comp, S.up[si], 0));
        rc = fe3d_quad4_kc0(n, d_cdof, d_iota, d_x, nx, nullptr, 0, nullptr, nullptr, nullptr, nullptr,
                            pid ? d_props : d_pset, pid ? nprops : n, pid ? d_pid : nullptr,
                            values_only ? nullptr : d_kr, values_only ? nullptr : d_kc, d_kv, ns, values_only,
                            d_err, comp);
        if (rc) break;
        FE3D_CUDA(cudaEventRecord(S.done[si], comp));
        // download
        FE3D_CUDA(cudaStreamWaitEvent(down, S.done[si], 0));
        FE3D_CUDA(cudaMemcpyAsync(Kv + s0, d_kv, sizeof(double) * ns, cudaMemcpyDeviceToHost, down));
        FE3D_CUDA(cudaEventRecord(S.down[si], down));
        FE3D_CUDA(cudaStreamWaitEvent(down2, S.done[si], 0));
        if (!values_only) {
            FE3D_CUDA(cudaMemcpyAsync(Kr + s0, d_kr, sizeof(int64_t) * ns, cudaMemcpyDeviceToHost, down2));
            FE3D_CUDA(cudaMemcpyAsync(Kc + s0, d_kc, sizeof(int64_t) * ns, cudaMemcpyDeviceToHost, down2));
        }
        FE3D_CUDA(cudaEventRecord(S.down2[si], down2));
        e0 += n;
        if (want < chunk) want = 2 * want < chunk ? 2 * want : chunk;
    }
    int herr = 0;
    if (cudaStreamSynchronize(comp) != cudaSuccess || cudaStreamSynchronize(down) != cudaSuccess ||
        cudaStreamSynchronize(down2) != cudaSuccess ||
        cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return rc ? rc : FE3D_ERR_CUDA;
    if (rc) return rc;
    if (err_host) *err_host |= herr;
    return FE3D_OK;
}
