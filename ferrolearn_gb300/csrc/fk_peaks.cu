// fk_peaks.cu -- CUDA-core throughput microbenchmarks for the roofline of the
// SIMT kernels (the measured peaks file holds only HBM copy bandwidth and BF16
// tensor throughput). Each thread runs eight independent chains of one operation;
// rates are counted per operation executed (an FMA counts as two flops).
#include "fk_internal.cuh"

namespace fk {
namespace {

constexpr int CHAINS = 8;

template <typename T, int OP>
__global__ void peak_kernel(T a, T b, int iters, T *out) {
    T acc[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; c++) acc[c] = (T)(threadIdx.x + c);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
#pragma unroll
            for (int c = 0; c < CHAINS; c++) {
                if (OP == 0) acc[c] = acc[c] * a + b;  // fused multiply-add
                else acc[c] = acc[c] + a;              // add only
            }
        }
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; c++) s += acc[c];
    if (s == (T)-1.2345) out[threadIdx.x] = s;  // keeps the chains alive
}

// One dependent chain per thread, one warp per SM: the latency of the op.
template <typename T>
__global__ void latency_kernel(T a, int iters, T *out, long long *cycles) {
    T acc = (T)threadIdx.x;
    long long t0 = clock64();
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) acc = acc + a;
    }
    long long t1 = clock64();
    if (threadIdx.x == 0 && blockIdx.x == 0) *cycles = t1 - t0;
    if (acc == (T)-1.2345) out[threadIdx.x] = acc;
}

template <typename T, int OP>
double time_peak(Ctx &ctx, int iters) {
    T *out = (T *)ctx.get(BUF_OUT, 4096 * sizeof(T));
    const int blocks = ctx.num_sms * 4, threads = 256;
    peak_kernel<T, OP><<<blocks, threads, 0, ctx.stream>>>((T)1.0000001, (T)0.5, 2, out);
    FK_LAUNCH_CHECK();
    Events<2> ev;
    FK_CUDA(cudaEventRecord(ev[0], ctx.stream));
    peak_kernel<T, OP><<<blocks, threads, 0, ctx.stream>>>((T)1.0000001, (T)0.5, iters, out);
    FK_LAUNCH_CHECK();
    FK_CUDA(cudaEventRecord(ev[1], ctx.stream));
    FK_CUDA(cudaEventSynchronize(ev[1]));
    float ms = 0.f;
    FK_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    const double ops = (double)blocks * threads * iters * 16.0 * CHAINS * (OP == 0 ? 2.0 : 1.0);
    return ops / (ms * 1e-3);
}

}  // namespace

// out: [0] FP32 FMA flop/s, [1] FP64 FMA flop/s, [2] FP64 add op/s,
//      [3] FP32 add op/s, [4] FP64 add latency (cycles), [5] FP32 add latency
void measure_peaks(Ctx &ctx, double *out) {
    out[0] = time_peak<float, 0>(ctx, 4096);
    out[1] = time_peak<double, 0>(ctx, 256);
    out[2] = time_peak<double, 1>(ctx, 256);
    out[3] = time_peak<float, 1>(ctx, 4096);
    long long *cyc = (long long *)ctx.get(BUF_OUT2, 64);
    double *od = (double *)ctx.get(BUF_OUT, 4096 * sizeof(double));
    long long h = 0;
    latency_kernel<double><<<1, 32, 0, ctx.stream>>>(1.0000001, 256, od, cyc);
    FK_LAUNCH_CHECK();
    FK_CUDA(cudaMemcpyAsync(&h, cyc, sizeof(h), cudaMemcpyDeviceToHost, ctx.stream));
    FK_CUDA(cudaStreamSynchronize(ctx.stream));
    out[4] = (double)h / (256.0 * 16.0);
    latency_kernel<float><<<1, 32, 0, ctx.stream>>>(1.0000001f, 256, (float *)od, cyc);
    FK_LAUNCH_CHECK();
    FK_CUDA(cudaMemcpyAsync(&h, cyc, sizeof(h), cudaMemcpyDeviceToHost, ctx.stream));
    FK_CUDA(cudaStreamSynchronize(ctx.stream));
    out[5] = (double)h / (256.0 * 16.0);
}

}  // namespace fk
