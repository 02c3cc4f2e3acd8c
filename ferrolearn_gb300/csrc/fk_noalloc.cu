// fk_noalloc.cu -- an assignment + inertia entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc at the moment they need a KMeans score:
// code running between the steps of a latency-critical serving loop (an
// allocation can synchronise the whole device), code working under a fixed
// memory budget that has already been handed out, or hosts whose allocator
// is owned by another framework. fk_kmeans_score_f64_noalloc serves them: the
// caller passes device buffers for the inputs and the outputs, and the only
// scratch the computation needs -- the per-row nearest-centre labels and
// minimum distances, and the partial sums of the fixed-order inertia
// reduction -- lives in one file-scope __device__ array of fixed size that
// every GPU loading this library holds until the process exits.
//
// The arithmetic is the plain FP64 path's: direct-form distances with the
// lowest index on ties (kmeans.rs:159-163, 295-309) and the inertia as the
// same fixed-order f64 tree as fk_lloyd_step_f64 uses for its sum.
#include <mutex>

#include "fk_internal.cuh"

namespace fk {
namespace {

// Capacity of the shared scratch: 524,288 rows (12 bytes per row: an int32
// label and an f64 distance) plus the partial sums -- about 6.3 MB per GPU.
constexpr int64_t NOALLOC_MAX_ROWS = 1 << 19;
constexpr size_t NOALLOC_PARTIALS = 1024;
constexpr size_t NOALLOC_OFF_MIND = 0;
constexpr size_t NOALLOC_OFF_LABELS = NOALLOC_OFF_MIND + sizeof(double) * NOALLOC_MAX_ROWS;
constexpr size_t NOALLOC_OFF_PARTIALS = NOALLOC_OFF_LABELS + sizeof(int32_t) * NOALLOC_MAX_ROWS;
constexpr size_t NOALLOC_BYTES = NOALLOC_OFF_PARTIALS + sizeof(double) * NOALLOC_PARTIALS;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Device address of g_noalloc_scratch, looked up once per device (the host
// name of the array is only a stand-in, never a device address). The address
// belongs to the device's primary context, the one the CUDA runtime uses: the
// entry point must be called with that context current, and after
// cudaDeviceReset (which destroys it) the cached address is stale, so a
// process that resets a device must not call this entry point on it again.
constexpr int NOALLOC_MAX_DEVICES = 64;
void *g_scratch_addr[NOALLOC_MAX_DEVICES] = {};
std::mutex g_scratch_mu;

void *scratch_for_current_device() {
    int dev = 0;
    FK_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        set_error("device %d is beyond the %d devices the allocation-free entry point tracks", dev,
                  NOALLOC_MAX_DEVICES);
        fail(FK_ERR_UNSUPPORTED);
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error("cudaGetSymbolAddress of the scratch array failed on device %d: %s", dev,
                      cudaGetErrorString(e));
            fail(FK_ERR_CUDA);
        }
        g_scratch_addr[dev] = p;
    }
    return g_scratch_addr[dev];
}

// Device memory of the current GPU (or managed memory). A buffer on another
// GPU is refused here: without peer access the kernels would fault on it.
bool on_device(const void *p, const char *name) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        set_error("`%s` is not device memory: every buffer passed to the allocation-free entry point must be",
                  name);
        return false;
    }
    if (a.type == cudaMemoryTypeDevice) {
        int cur = 0;
        FK_CUDA(cudaGetDevice(&cur));
        if (a.device != cur) {
            set_error("`%s` is device memory of GPU %d, but the current GPU is %d", name, a.device, cur);
            return false;
        }
        return true;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    set_error("`%s` is not device memory: every buffer passed to the allocation-free entry point must be", name);
    return false;
}

}  // namespace
}  // namespace fk

extern "C" fk_status fk_kmeans_score_f64_noalloc(const double *x, int64_t n, int64_t d, const double *centers,
                                                 int64_t k, uint64_t *labels_out, double *inertia_out,
                                                 void *cuda_stream) {
    using namespace fk;
    try {
        if (!x || !centers || !labels_out || !inertia_out) {
            set_error("required pointer is NULL");
            return FK_ERR_NULL_POINTER;
        }
        if (k <= 0) {
            set_error("Invalid parameter `n_clusters`: must be at least 1");
            return FK_ERR_INVALID_PARAMETER;
        }
        if (n <= 0 || d < 0) {
            set_error("Invalid parameter: n must be at least 1 and d non-negative");
            return FK_ERR_INVALID_PARAMETER;
        }
        if (n > NOALLOC_MAX_ROWS) {
            set_error("n = %lld rows exceeds the allocation-free scratch capacity of %lld rows; "
                      "use fk_lloyd_step_f64 / fk_kmeans_predict_f64 instead",
                      (long long)n, (long long)NOALLOC_MAX_ROWS);
            return FK_ERR_INVALID_PARAMETER;
        }
        if (k > INT32_MAX || d > (1 << 16)) {
            set_error("shape d=%lld k=%lld exceeds the supported range", (long long)d, (long long)k);
            return FK_ERR_UNSUPPORTED;
        }
        if (!on_device(x, "x") || !on_device(centers, "centers") || !on_device(labels_out, "labels_out") ||
            !on_device(inertia_out, "inertia_out"))
            return FK_ERR_INVALID_PARAMETER;
        unsigned char *base = (unsigned char *)scratch_for_current_device();
        double *mind = (double *)(base + NOALLOC_OFF_MIND);
        int32_t *labels = (int32_t *)(base + NOALLOC_OFF_LABELS);
        double *partials = (double *)(base + NOALLOC_OFF_PARTIALS);
        cudaStream_t s = (cudaStream_t)cuda_stream;
        // Every scratch value read below is written earlier in the same call
        // (labels, distances, then partials), so nothing needs clearing.
        launch_assign_direct<double, double>(x, n, (int)d, centers, (int)k, labels, mind, s);
        launch_labels_to_u64(labels, n, labels_out, s);
        launch_sum_fixed<double>(mind, n, partials, inertia_out, s);
        return FK_OK;
    } catch (const Error &e) {
        return e.code;
    } catch (...) {
        set_error("unexpected exception");
        return FK_ERR_CUDA;
    }
}
