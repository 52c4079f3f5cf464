// C ABI (include/pcbqs_gb300.h): device context, geometry upload, and the fill / combine / potential entry points.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <new>
#include <type_traits>
#include <string>
#include <vector>

#include "../../include/pcbqs_gb300.h"
#include "combine.cuh"
#include "common.cuh"
#include "fill.cuh"

using namespace pq;

namespace {
thread_local std::string g_error;
std::atomic<long long> g_launches{0};
std::atomic<unsigned long long> g_wait_cycles{0};
}  // namespace

void pq::note_launches(long long count) { g_launches.fetch_add(count, std::memory_order_relaxed); }

unsigned long long pq::wait_cycles() {
    const unsigned long long w = g_wait_cycles.load(std::memory_order_relaxed);
    return w ? w : DEFAULT_WAIT_CYCLES;
}

extern "C" int pcbqs_gb300_set_wait_cycles(uint64_t cycles) {
    g_wait_cycles.store(cycles, std::memory_order_relaxed);
    return OK;
}

// The calling thread's last error message, shared by every entry point of the library.
int pq::fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_error = buf;
    return code;
}

namespace {

int cuda_fail(cudaError_t err, const char *what) {
    return fail(ERR_CUDA, "%s: %s", what, cudaGetErrorString(err));
}

#define CK(call)                                              \
    do {                                                      \
        cudaError_t err_ = (call);                            \
        if (err_ != cudaSuccess) return cuda_fail(err_, #call); \
    } while (0)

// One device allocation that is released when the owner goes away.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t n) {
        if (n <= bytes) return cudaSuccess;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        cudaError_t err = cudaMalloc(&ptr, n);
        if (err == cudaSuccess) bytes = n;
        return err;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
};

}  // namespace

struct pcbqs_gb300_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    Geometry g{};
    DevBuf geometry;        // FarRec, ClsRec, SrcRec records and observation rules
    DevBuf flags;           // [0] non-finite, [1] status, then 8 counters (64-bit)
    DevBuf near_lists;      // two int2 lists
    unsigned long long near_capacity = 0;
    DevBuf pair_io;         // pair-list staging (host entry point)
    DevBuf planes;          // device moment planes (host fill entry point)
    size_t planes_ld = 0;
    uint64_t last_counts[2] = {0, 0};   // near pairs of the last fill: level 0, level `outer`
};

namespace {

struct DeviceGuard {
    int previous = -1;
    explicit DeviceGuard(int device) {
        cudaGetDevice(&previous);
        if (previous != device) cudaSetDevice(device);
    }
    ~DeviceGuard() {
        int now = -1;
        cudaGetDevice(&now);
        if (previous >= 0 && now != previous) cudaSetDevice(previous);
    }
};

int *flag_ptr(pcbqs_gb300_ctx *c) { return static_cast<int *>(c->flags.ptr); }
unsigned long long *counter_ptr(pcbqs_gb300_ctx *c) {
    return reinterpret_cast<unsigned long long *>(static_cast<char *>(c->flags.ptr) + 16);
}

int read_flags(pcbqs_gb300_ctx *c, cudaStream_t stream, int *host2) {
    CK(cudaMemcpyAsync(host2, c->flags.ptr, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    return OK;
}

}  // namespace

// The device geometry of a context, for the other kernels of the library (hmatrix.cu).
const Geometry *pcbqs_gb300_geometry_of(const pcbqs_gb300_ctx *ctx) { return &ctx->g; }

extern "C" {

const char *pcbqs_gb300_last_error(void) { return g_error.c_str(); }

int64_t pcbqs_gb300_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int pcbqs_gb300_fill_counts(const pcbqs_gb300_ctx *c, uint64_t *counts) {
    if (!c || !counts) return fail(ERR_ARGUMENT, "fill_counts: null argument");
    counts[0] = c->last_counts[0];
    counts[1] = c->last_counts[1];
    return OK;
}

int32_t pcbqs_gb300_triangles(const pcbqs_gb300_ctx *ctx) { return ctx ? ctx->g.nt : 0; }

int pcbqs_gb300_create(const pcbqs_gb300_geometry *geo, int device, pcbqs_gb300_ctx **out) {
    if (!geo || !out) return fail(ERR_ARGUMENT, "create: null geometry or output");
    *out = nullptr;
    const int nt = geo->nt;
    if (nt <= 0) return fail(ERR_ARGUMENT, "create: no triangles");
    if (!geo->v || !geo->len || !geo->tau || !geo->un || !geo->area || !geo->p3 || !geo->cent || !geo->radius ||
        !geo->z)
        return fail(ERR_ARGUMENT, "create: missing geometry array");
    for (int k = 0; k < 3; ++k)
        if (!geo->qp[k] || !geo->qw[k] || geo->nq[k] <= 0 || geo->nq[k] > 6 * 64)
            return fail(ERR_ARGUMENT, "create: invalid observation rule of level %d", k);
    int count = 0;
    cudaError_t err = cudaGetDeviceCount(&count);
    if (err != cudaSuccess || count <= 0) return fail(ERR_CUDA, "create: no CUDA device available (%s)",
                                                      cudaGetErrorString(err));
    if (device < 0 || device >= count) return fail(ERR_ARGUMENT, "create: device %d out of range", device);
    DeviceGuard guard(device);
    auto *c = new (std::nothrow) pcbqs_gb300_ctx();
    if (!c) return fail(ERR_MEMORY, "create: host allocation failed");
    c->device = device;
    err = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (err != cudaSuccess) {
        delete c;
        return cuda_fail(err, "cudaStreamCreate");
    }
    // Pack the host arrays into per-triangle records.
    std::vector<FarRec> far(nt);
    std::vector<ClsRec> cls(nt);
    std::vector<SrcRec> src(nt);
    std::vector<LocalRec> local(nt);
    for (int t = 0; t < nt; ++t) {
        const double cx = geo->cent[2 * (size_t)t], cy = geo->cent[2 * (size_t)t + 1];
        LocalRec &lr = local[t];
        lr.chi[0] = (float)cx;
        lr.chi[1] = (float)cy;
        lr.clo[0] = (float)(cx - (double)lr.chi[0]);
        lr.clo[1] = (float)(cy - (double)lr.chi[1]);
        for (int j = 0; j < 3; ++j) {
            lr.u[2 * j] = (float)(geo->p3[6 * (size_t)t + 2 * j] - cx);
            lr.u[2 * j + 1] = (float)(geo->p3[6 * (size_t)t + 2 * j + 1] - cy);
        }
        lr.area = (float)geo->area[t];
        lr.z = (float)geo->z[t];
        for (int j = 0; j < 6; ++j) far[t].p[j] = geo->p3[6 * (size_t)t + j];
        far[t].area = geo->area[t];
        far[t].z = geo->z[t];
        cls[t] = ClsRec{geo->cent[2 * (size_t)t], geo->cent[2 * (size_t)t + 1], geo->radius[t], geo->z[t]};
        for (int j = 0; j < 6; ++j) {
            src[t].v[j] = geo->v[6 * (size_t)t + j];
            src[t].tau[j] = geo->tau[6 * (size_t)t + j];
            src[t].un[j] = geo->un[6 * (size_t)t + j];
        }
        for (int j = 0; j < 3; ++j) src[t].len[j] = geo->len[3 * (size_t)t + j];
        src[t].area = geo->area[t];
        src[t].pad[0] = src[t].pad[1] = 0;
    }
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t off_far = 0, off_cls = up(off_far + sizeof(FarRec) * (size_t)nt);
    const size_t off_src = up(off_cls + sizeof(ClsRec) * (size_t)nt);
    const size_t off_loc = up(off_src + sizeof(SrcRec) * (size_t)nt);
    size_t off = off_loc + sizeof(LocalRec) * (size_t)nt;
    size_t off_obs[3], off_w[3];
    for (int k = 0; k < 3; ++k) {
        off = up(off);
        off_obs[k] = off;
        off += sizeof(double) * 2 * (size_t)nt * geo->nq[k];
        off = up(off);
        off_w[k] = off;
        off += sizeof(double) * geo->nq[k];
    }
    err = c->geometry.reserve(off);
    if (err == cudaSuccess) err = c->flags.reserve(256);
    if (err != cudaSuccess) {
        c->geometry.release();
        c->flags.release();
        cudaStreamDestroy(c->stream);
        delete c;
        return fail(ERR_MEMORY, "create: device allocation of %zu bytes failed: %s", off, cudaGetErrorString(err));
    }
    char *base = static_cast<char *>(c->geometry.ptr);
    auto put = [&](size_t at, const void *src_ptr, size_t bytes) {
        return cudaMemcpyAsync(base + at, src_ptr, bytes, cudaMemcpyHostToDevice, c->stream);
    };
    err = put(off_far, far.data(), sizeof(FarRec) * (size_t)nt);
    if (err == cudaSuccess) err = put(off_cls, cls.data(), sizeof(ClsRec) * (size_t)nt);
    if (err == cudaSuccess) err = put(off_src, src.data(), sizeof(SrcRec) * (size_t)nt);
    if (err == cudaSuccess) err = put(off_loc, local.data(), sizeof(LocalRec) * (size_t)nt);
    for (int k = 0; k < 3 && err == cudaSuccess; ++k) {
        err = put(off_obs[k], geo->qp[k], sizeof(double) * 2 * (size_t)nt * geo->nq[k]);
        if (err == cudaSuccess) err = put(off_w[k], geo->qw[k], sizeof(double) * geo->nq[k]);
    }
    if (err == cudaSuccess) err = cudaMemsetAsync(c->flags.ptr, 0, 256, c->stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(c->stream);
    if (err != cudaSuccess) {
        pcbqs_gb300_destroy(c);
        return cuda_fail(err, "create: geometry upload");
    }
    c->g.nt = nt;
    c->g.far = reinterpret_cast<const FarRec *>(base + off_far);
    c->g.cls = reinterpret_cast<const ClsRec *>(base + off_cls);
    c->g.src = reinterpret_cast<const SrcRec *>(base + off_src);
    c->g.local = reinterpret_cast<const LocalRec *>(base + off_loc);
    for (int k = 0; k < 3; ++k) {
        c->g.obs[k] = reinterpret_cast<const double *>(base + off_obs[k]);
        c->g.w[k] = reinterpret_cast<const double *>(base + off_w[k]);
        c->g.nq[k] = geo->nq[k];
    }
    *out = c;
    return OK;
}

void pcbqs_gb300_destroy(pcbqs_gb300_ctx *c) {
    if (!c) return;
    DeviceGuard guard(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->geometry.release();
    c->flags.release();
    c->near_lists.release();
    c->pair_io.release();
    c->planes.release();
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

static int pairs_on_device(pcbqs_gb300_ctx *c, const int32_t *p, const int32_t *q, const double *d,
                           const int32_t *kind, int64_t n, int scalar_only, double *out, int64_t *order,
                           cudaStream_t stream) {
    CK(cudaMemsetAsync(c->flags.ptr, 0, 2 * sizeof(int), stream));
    CK(launch_pairs(c->g, p, q, d, kind, n, scalar_only, out, counter_ptr(c), order, flag_ptr(c), flag_ptr(c) + 1,
                    stream));
    int host[2];
    int rc = read_flags(c, stream, host);
    if (rc) return rc;
    if (host[1]) return fail(ERR_ARGUMENT, "pairs: triangle index or kind out of range");
    if (host[0]) return fail(ERR_NONFINITE, "non-finite triangle-pair moments from fill backend");
    return OK;
}

int pcbqs_gb300_pairs(pcbqs_gb300_ctx *c, const int32_t *p, const int32_t *q, const double *d, const int32_t *kind,
                      int64_t n, int scalar_only, double *out) {
    if (!c) return fail(ERR_ARGUMENT, "pairs: null context");
    if (n < 0) return fail(ERR_ARGUMENT, "pairs: negative count");
    if (n == 0) return OK;
    if (!p || !q || !d || !kind || !out) return fail(ERR_ARGUMENT, "pairs: null array");
    const int nt = c->g.nt;
    for (int64_t i = 0; i < n; ++i) {
        if (p[i] < 0 || p[i] >= nt || q[i] < 0 || q[i] >= nt)
            return fail(ERR_ARGUMENT, "pairs: triangle index out of range at %lld", (long long)i);
        if (kind[i] < -1 || kind[i] > 2) return fail(ERR_ARGUMENT, "pairs: invalid kind at %lld", (long long)i);
        if (!std::isfinite(d[i])) return fail(ERR_ARGUMENT, "pairs: non-finite offset at %lld", (long long)i);
    }
    DeviceGuard guard(c->device);
    const int width = scalar_only ? 1 : 6;
    const size_t b_idx = sizeof(int32_t) * (size_t)n, b_d = sizeof(double) * (size_t)n;
    const size_t b_out = sizeof(double) * (size_t)n * width, b_ord = sizeof(int64_t) * (size_t)n;
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t o_p = 0, o_q = align(b_idx), o_k = o_q + align(b_idx), o_d = o_k + align(b_idx);
    const size_t o_out = o_d + align(b_d), o_ord = o_out + align(b_out), total = o_ord + align(b_ord);
    cudaError_t err = c->pair_io.reserve(total);
    if (err != cudaSuccess) return fail(ERR_MEMORY, "pairs: device allocation failed: %s", cudaGetErrorString(err));
    char *base = static_cast<char *>(c->pair_io.ptr);
    cudaStream_t s = c->stream;
    CK(cudaMemcpyAsync(base + o_p, p, b_idx, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_q, q, b_idx, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_k, kind, b_idx, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_d, d, b_d, cudaMemcpyHostToDevice, s));
    int rc = pairs_on_device(c, reinterpret_cast<int32_t *>(base + o_p), reinterpret_cast<int32_t *>(base + o_q),
                             reinterpret_cast<double *>(base + o_d), reinterpret_cast<int32_t *>(base + o_k), n,
                             scalar_only, reinterpret_cast<double *>(base + o_out),
                             reinterpret_cast<int64_t *>(base + o_ord), s);
    if (rc) return rc;
    CK(cudaMemcpyAsync(out, base + o_out, b_out, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return OK;
}

int pcbqs_gb300_pairs_device(pcbqs_gb300_ctx *c, const int32_t *p, const int32_t *q, const double *d,
                             const int32_t *kind, int64_t n, int scalar_only, double *out, void *stream) {
    if (!c) return fail(ERR_ARGUMENT, "pairs_device: null context");
    if (n < 0) return fail(ERR_ARGUMENT, "pairs_device: negative count");
    if (n == 0) return OK;
    DeviceGuard guard(c->device);
    cudaError_t err = c->pair_io.reserve(sizeof(int64_t) * (size_t)n);
    if (err != cudaSuccess) return fail(ERR_MEMORY, "pairs_device: device allocation failed");
    return pairs_on_device(c, p, q, d, kind, n, scalar_only, out, static_cast<int64_t *>(c->pair_io.ptr),
                           static_cast<cudaStream_t>(stream));
}

}  // extern "C"

// Fill into device planes; lists grow (and the fill reruns) when the near pairs outnumber their capacity.
// T = double: the reference's FP64 moments; T = float: mixed precision, moments about each triangle's centroid.
template <class T>
static int fill_device(pcbqs_gb300_ctx *c, double near, int outer, int scalar_only, T *const *planes,
                       int64_t ld, uint64_t *analytic, cudaStream_t stream) {
    const int nt = c->g.nt;
    if (outer < 0 || outer > 2) return fail(ERR_ARGUMENT, "fill: outer_levels must be 0, 1 or 2");
    if (std::isnan(near)) return fail(ERR_ARGUMENT, "fill: near must be nonnegative (or infinity)");
    if (ld < nt) return fail(ERR_ARGUMENT, "fill: leading dimension %lld below %d", (long long)ld, nt);
    if (!planes || !planes[0] || (!scalar_only && (!planes[1] || !planes[2] || !planes[3])))
        return fail(ERR_ARGUMENT, "fill: missing output plane");
    FillRule rule{near, (near < 0 || std::isinf(near)) ? 1 : 0, outer, wait_cycles()};
    if (rule.all_near) rule.near = 0;
    Planes<T> fp{planes[0], scalar_only ? nullptr : planes[1], scalar_only ? nullptr : planes[2],
                 scalar_only ? nullptr : planes[3], ld, scalar_only};
    constexpr bool local = std::is_same<T, float>::value;
    const unsigned long long pairs = (unsigned long long)nt * (nt + 1) / 2;
    if (!c->near_capacity) {
        unsigned long long guess = std::max<unsigned long long>(1ull << 16, pairs / 16);
        c->near_capacity = std::min(guess, pairs);
    }
    for (int attempt = 0; attempt < 2; ++attempt) {
        cudaError_t err = c->near_lists.reserve(2 * sizeof(int2) * c->near_capacity);
        if (err != cudaSuccess)
            return fail(ERR_MEMORY, "fill: near-pair lists of %llu entries: %s", c->near_capacity,
                        cudaGetErrorString(err));
        NearLists lists{{static_cast<int2 *>(c->near_lists.ptr),
                         static_cast<int2 *>(c->near_lists.ptr) + c->near_capacity},
                        counter_ptr(c),
                        c->near_capacity};
        CK(cudaMemsetAsync(c->flags.ptr, 0, 2 * sizeof(int), stream));
        if constexpr (local) CK(launch_fill_local(c->g, fp, rule, lists, flag_ptr(c), flag_ptr(c) + 1, stream));
        else CK(launch_fill(c->g, fp, rule, lists, flag_ptr(c), flag_ptr(c) + 1, stream));
        unsigned long long counts[2];
        CK(cudaMemcpyAsync(counts, lists.count, sizeof counts, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        if (std::max(counts[0], counts[1]) > c->near_capacity) {
            c->near_capacity = std::min(pairs, std::max(counts[0], counts[1]) + (1ull << 12));
            continue;
        }
        if constexpr (local) CK(launch_fill_near_local(c->g, fp, rule, lists, flag_ptr(c), stream));
        else CK(launch_fill_near(c->g, fp, rule, lists, flag_ptr(c), stream));
        int host[2];
        int rc = read_flags(c, stream, host);
        if (rc) return rc;
        if (host[1]) return fail(host[1], "fill: a bounded wait for staged geometry gave up");
        if (host[0]) return fail(ERR_NONFINITE, "non-finite triangle-pair moments from fill backend");
        if (analytic) *analytic = counts[0] + (rule.outer ? counts[1] : 0);
        c->last_counts[0] = counts[0];
        c->last_counts[1] = rule.outer ? counts[1] : 0;
        return OK;
    }
    return fail(ERR_MEMORY, "fill: near-pair lists did not fit");
}

extern "C" {

int pcbqs_gb300_fill_device(pcbqs_gb300_ctx *c, double near, int outer, int scalar_only, double *const *planes,
                            int64_t ld, uint64_t *analytic, void *stream) {
    if (!c) return fail(ERR_ARGUMENT, "fill_device: null context");
    DeviceGuard guard(c->device);
    return fill_device<double>(c, near, outer, scalar_only, planes, ld, analytic, static_cast<cudaStream_t>(stream));
}

int pcbqs_gb300_fill_local_device(pcbqs_gb300_ctx *c, double near, int outer, int scalar_only, float *const *planes,
                                  int64_t ld, uint64_t *analytic, void *stream) {
    if (!c) return fail(ERR_ARGUMENT, "fill_local_device: null context");
    DeviceGuard guard(c->device);
    return fill_device<float>(c, near, outer, scalar_only, planes, ld, analytic, static_cast<cudaStream_t>(stream));
}

int pcbqs_gb300_fill(pcbqs_gb300_ctx *c, double near, int outer, int scalar_only, double *const *planes,
                     uint64_t *analytic) {
    if (!c) return fail(ERR_ARGUMENT, "fill: null context");
    if (!planes || !planes[0] || (!scalar_only && (!planes[1] || !planes[2] || !planes[3])))
        return fail(ERR_ARGUMENT, "fill: missing output plane");
    DeviceGuard guard(c->device);
    const int nt = c->g.nt;
    const int width = scalar_only ? 1 : 4;
    const size_t plane = (size_t)nt * nt;
    cudaError_t err = c->planes.reserve(sizeof(double) * plane * width);
    if (err != cudaSuccess)
        return fail(ERR_MEMORY, "fill: %d device planes of %d x %d: %s", width, nt, nt, cudaGetErrorString(err));
    double *dev[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int k = 0; k < width; ++k) dev[k] = static_cast<double *>(c->planes.ptr) + k * plane;
    int rc = fill_device<double>(c, near, outer, scalar_only, dev, nt, analytic, c->stream);
    if (rc) return rc;
    for (int k = 0; k < width; ++k)
        CK(cudaMemcpyAsync(planes[k], dev[k], sizeof(double) * plane, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return OK;
}

int pcbqs_gb300_edge_inductance_device(int64_t ne, const int32_t *tri, const double *alpha, const double *vertex,
                                       const double *scale, double factor, const double *mrr, const double *mx,
                                       const double *my, const double *m0, int64_t ldm, double *L, int64_t ldl,
                                       void *stream) {
    if (ne < 0 || ldl < ne) return fail(ERR_ARGUMENT, "edge_inductance: invalid sizes");
    if (ne == 0) return OK;
    if (!tri || !alpha || !vertex || !scale || !mrr || !mx || !my || !m0 || !L)
        return fail(ERR_ARGUMENT, "edge_inductance: null array");
    EdgeBasis e{ne, tri, alpha, vertex, scale};
    MomentPlanes mo{m0, mx, my, mrr, ldm};
    CK(launch_edge_inductance(e, mo, factor, L, ldl, static_cast<cudaStream_t>(stream)));
    return OK;
}

int pcbqs_gb300_edge_inductance(int64_t nt, int64_t ne, const int32_t *tri, const double *alpha,
                                const double *vertex, const double *scale, double factor, const double *mrr,
                                const double *mx, const double *my, const double *m0, double *L) {
    if (nt <= 0 || ne < 0) return fail(ERR_ARGUMENT, "edge_inductance: invalid sizes");
    if (ne == 0) return OK;
    for (int64_t i = 0; i < 2 * ne; ++i)
        if (tri[i] < 0 || tri[i] >= nt) return fail(ERR_ARGUMENT, "edge_inductance: invalid triangle index");
    const size_t plane = (size_t)nt * nt, lbytes = sizeof(double) * (size_t)ne * ne;
    const size_t b_tri = sizeof(int32_t) * 2 * ne, b_al = sizeof(double) * 2 * ne, b_v = sizeof(double) * 4 * ne,
                 b_s = sizeof(double) * ne;
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t o_m = 0, o_l = o_m + align(4 * sizeof(double) * plane), o_t = o_l + align(lbytes);
    const size_t o_a = o_t + align(b_tri), o_v = o_a + align(b_al), o_s = o_v + align(b_v), total = o_s + align(b_s);
    DevBuf buf;
    cudaError_t err = buf.reserve(total);
    if (err != cudaSuccess) return fail(ERR_MEMORY, "edge_inductance: device allocation failed");
    char *base = static_cast<char *>(buf.ptr);
    double *dm = reinterpret_cast<double *>(base + o_m);
    cudaStream_t s = nullptr;
    int rc = OK;
    const double *src[4] = {m0, mx, my, mrr};
    for (int k = 0; k < 4 && rc == OK; ++k)
        if ((err = cudaMemcpyAsync(dm + k * plane, src[k], sizeof(double) * plane, cudaMemcpyHostToDevice, s)))
            rc = cuda_fail(err, "edge_inductance: upload");
    if (rc == OK && ((err = cudaMemcpyAsync(base + o_t, tri, b_tri, cudaMemcpyHostToDevice, s)) ||
                     (err = cudaMemcpyAsync(base + o_a, alpha, b_al, cudaMemcpyHostToDevice, s)) ||
                     (err = cudaMemcpyAsync(base + o_v, vertex, b_v, cudaMemcpyHostToDevice, s)) ||
                     (err = cudaMemcpyAsync(base + o_s, scale, b_s, cudaMemcpyHostToDevice, s))))
        rc = cuda_fail(err, "edge_inductance: upload");
    if (rc == OK)
        rc = pcbqs_gb300_edge_inductance_device(ne, reinterpret_cast<int32_t *>(base + o_t),
                                                reinterpret_cast<double *>(base + o_a),
                                                reinterpret_cast<double *>(base + o_v),
                                                reinterpret_cast<double *>(base + o_s), factor, dm + 3 * plane,
                                                dm + plane, dm + 2 * plane, dm, nt,
                                                reinterpret_cast<double *>(base + o_l), ne, s);
    if (rc == OK && (err = cudaMemcpyAsync(L, base + o_l, lbytes, cudaMemcpyDeviceToHost, s)))
        rc = cuda_fail(err, "edge_inductance: download");
    if (rc == OK && (err = cudaStreamSynchronize(s))) rc = cuda_fail(err, "edge_inductance");
    buf.release();
    return rc;
}

int pcbqs_gb300_edge_inductance_local_device(int64_t ne, const int32_t *tri, const float *alpha, const float *off,
                                             const float *scale, double factor, const float *mrr, const float *mx,
                                             const float *my, const float *m0, int64_t ldm, double *L, int64_t ldl,
                                             float *Lf, int64_t ldlf, void *stream) {
    if (ne < 0 || ldl < ne || (Lf && ldlf < ne)) return fail(ERR_ARGUMENT, "edge_inductance_local: invalid sizes");
    if (ne == 0) return OK;
    if (!tri || !alpha || !off || !scale || !mrr || !mx || !my || !m0 || !L)
        return fail(ERR_ARGUMENT, "edge_inductance_local: null array");
    EdgeBasisF e{ne, tri, alpha, off, scale};
    MomentPlanesF mo{m0, mx, my, mrr, ldm};
    CK(launch_edge_inductance_local(e, mo, (float)factor, L, ldl, Lf, ldlf, static_cast<cudaStream_t>(stream)));
    return OK;
}

int pcbqs_gb300_potential_single_device(int64_t nn, const int64_t *start, const int32_t *members, const double *area,
                                        const float *m0, int64_t ldm, double factor, double *P, float *Pf,
                                        int64_t ldp, void *stream) {
    if (nn < 0 || ldp < nn) return fail(ERR_ARGUMENT, "potential_single: invalid sizes");
    if (nn == 0) return OK;
    if (!start || !members || !area || !m0 || !P) return fail(ERR_ARGUMENT, "potential_single: null array");
    NodeGroups ng{nn, start, members, area};
    CK(launch_potential_single(ng, m0, ldm, factor, P, Pf, ldp, static_cast<cudaStream_t>(stream)));
    return OK;
}

int pcbqs_gb300_potential_device(int64_t nn, const int64_t *start, const int32_t *members, const double *area,
                                 const double *m0, int64_t ldm, double factor, double *P, int64_t ldp,
                                 void *stream) {
    if (nn < 0 || ldp < nn) return fail(ERR_ARGUMENT, "potential: invalid sizes");
    if (nn == 0) return OK;
    if (!start || !members || !area || !m0 || !P) return fail(ERR_ARGUMENT, "potential: null array");
    NodeGroups ng{nn, start, members, area};
    CK(launch_potential(ng, m0, ldm, factor, P, ldp, static_cast<cudaStream_t>(stream)));
    return OK;
}

}  // extern "C"

// ---- Pair evaluation without device allocation -----------------------------------------------------------------
//
// pcbqs_gb300_pairs_device grows a per-context buffer with cudaMalloc for the kind-sorted pair order. Some callers
// cannot let a library allocate at call time: an application whose caching allocator has already reserved the
// device memory (cudaMalloc then fails even though the memory is free in the application's pool), and a service
// that must not stall in steady state, since cudaMalloc and cudaFree can synchronize the device. For them,
// pcbqs_gb300_pairs_no_alloc keeps its scratch (the order array, the kind counters and the status flags) in one
// array of fixed size that is part of this library's device image: it exists on every device that loads the
// library, is never allocated or freed by a call, and limits one call to NOALLOC_MAX_PAIRS pairs.
//
// Set-up: the first call on a device looks up the array's device address on that device (cudaGetSymbolAddress,
// which also loads this module there). Every call then synchronizes its stream to read the status flags back into
// host memory, so no call can be captured into a CUDA graph.
//
// Sharing: every call on a device uses the same array, which still holds the previous call's contents. Each call
// clears the counters and flags before its kernels run; the order array is fully rewritten before it is read.
// Two calls whose work overlaps on the GPU (concurrent streams, or host threads calling at once) race on the array
// and give wrong results: serialize them.

namespace {

constexpr int64_t NOALLOC_MAX_PAIRS = int64_t(1) << 20;    // 8 MB of order entries

struct NoAllocScratch {
    unsigned long long counters[8];     // per-kind counts [0..3] and scatter cursors [4..7]
    int flags[2];                       // [0] a moment is not finite, [1] an index or kind is out of range
    int pad[46];                        // the order array starts 256 bytes in
    int64_t order[NOALLOC_MAX_PAIRS];
};
static_assert(offsetof(NoAllocScratch, order) == 256, "scratch header is 256 bytes");

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

constexpr int NOALLOC_DEVICES = 64;
std::mutex g_noalloc_mutex;
NoAllocScratch *g_noalloc_address[NOALLOC_DEVICES] = {};

// The scratch array's address on `device` (the current device), looked up on the first call there.
int noalloc_scratch(int device, NoAllocScratch **out) {
    if (device < 0 || device >= NOALLOC_DEVICES)
        return fail(ERR_ARGUMENT, "pairs_no_alloc: device %d beyond the %d supported", device, NOALLOC_DEVICES);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_address[device]) {
        void *ptr = nullptr;
        const cudaError_t err = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (err != cudaSuccess) return cuda_fail(err, "pairs_no_alloc: cudaGetSymbolAddress");
        g_noalloc_address[device] = static_cast<NoAllocScratch *>(ptr);
    }
    *out = g_noalloc_address[device];
    return OK;
}

}  // namespace

extern "C" int pcbqs_gb300_pairs_no_alloc(pcbqs_gb300_ctx *c, const int32_t *p, const int32_t *q, const double *d,
                                          const int32_t *kind, int64_t n, int scalar_only, double *out,
                                          void *stream) {
    if (!c) return fail(ERR_ARGUMENT, "pairs_no_alloc: null context");
    if (n < 0) return fail(ERR_ARGUMENT, "pairs_no_alloc: negative count");
    if (n > NOALLOC_MAX_PAIRS)
        return fail(ERR_ARGUMENT, "pairs_no_alloc: %lld pairs exceed the fixed scratch of %lld pairs per call",
                    (long long)n, (long long)NOALLOC_MAX_PAIRS);
    if (n == 0) return OK;
    if (!p || !q || !d || !kind || !out) return fail(ERR_ARGUMENT, "pairs_no_alloc: null array");
    DeviceGuard guard(c->device);
    NoAllocScratch *s = nullptr;
    int rc = noalloc_scratch(c->device, &s);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CK(cudaMemsetAsync(s, 0, offsetof(NoAllocScratch, order), st));     // counters and flags start at zero
    CK(launch_pairs(c->g, p, q, d, kind, n, scalar_only, out, s->counters, s->order, &s->flags[0], &s->flags[1],
                    st));
    int host[2];
    CK(cudaMemcpyAsync(host, s->flags, sizeof host, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (host[1]) return fail(ERR_ARGUMENT, "pairs_no_alloc: triangle index or kind out of range");
    if (host[0]) return fail(ERR_NONFINITE, "non-finite triangle-pair moments from fill backend");
    return OK;
}
