// Integer issue-rate microbenchmark: the measured denominator of the fill
// kernels' roofline.
//
// The fill is min-plus int32 DP with tie flags: its work is 32-bit adds,
// two- and three-way minima, compares and bit logic, all on the integer
// pipes. Each kernel here runs one of those instructions back to back on
// eight register chains per thread at full occupancy. Each result feeds two
// later instructions (x_i <- op(x_{i+1}, x_{i+2}) over a ring of eight), so
// no two consecutive operations can be folded into one three-input
// instruction, and six of every eight are independent (enough ILP to hide
// the pipe latency with 16 warps per scheduler).
//
// poyalgn_int32_peak reports thread-instructions per second of one kind;
// the roofline peak is the fastest single-operation kind (add, min or
// logic), so a kernel that reaches it on its algorithmic op count issues
// one op per lane per cycle of the fastest pipe.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pa_runtime.h"

namespace {

constexpr int CHAINS = 8;
constexpr int ROUNDS = 16;  // rounds of CHAINS instructions per loop trip

template <int OP>
__device__ __forceinline__ int op(int a, int b, int c)
{
    int r;
    if constexpr (OP == POYALGN_PEAK_ADD) {
        asm volatile("add.s32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    } else if constexpr (OP == POYALGN_PEAK_MIN) {
        asm volatile("min.s32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    } else if constexpr (OP == POYALGN_PEAK_LOGIC) {
        asm volatile("xor.b32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    } else if constexpr (OP == POYALGN_PEAK_MIN3) {
        r = __vimin3_s32(a, b, c);
    } else {
        static_assert(OP == POYALGN_PEAK_MAX3_U16X2, "op kind");
        r = (int)__vimax3_u16x2((unsigned)a, (unsigned)b, (unsigned)c);
    }
    return r;
}

template <int OP>
__global__ void __launch_bounds__(256) peak_kernel(int* sink, int iters, int seed)
{
    int x[CHAINS];
#pragma unroll
    for (int i = 0; i < CHAINS; i++) x[i] = seed * (i + 3) + (int)threadIdx.x * (2 * i + 1);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int r = 0; r < ROUNDS; r++) {
#pragma unroll
            for (int i = 0; i < CHAINS; i++)
                x[i] = op<OP>(x[(i + 1) % CHAINS], x[(i + 2) % CHAINS], x[(i + 3) % CHAINS]);
        }
    }
    int s = 0;
#pragma unroll
    for (int i = 0; i < CHAINS; i++) s ^= x[i];
    if (s == seed) sink[blockIdx.x] = s;  // keeps every chain live
}

template <int OP>
cudaError_t run(int grid, int iters, int seed, int* sink, cudaStream_t st)
{
    peak_kernel<OP><<<grid, 256, 0, st>>>(sink, iters, seed);
    return cudaGetLastError();
}

cudaError_t launch(int kind, int grid, int iters, int seed, int* sink, cudaStream_t st)
{
    switch (kind) {
    case POYALGN_PEAK_ADD: return run<POYALGN_PEAK_ADD>(grid, iters, seed, sink, st);
    case POYALGN_PEAK_MIN: return run<POYALGN_PEAK_MIN>(grid, iters, seed, sink, st);
    case POYALGN_PEAK_LOGIC: return run<POYALGN_PEAK_LOGIC>(grid, iters, seed, sink, st);
    case POYALGN_PEAK_MIN3: return run<POYALGN_PEAK_MIN3>(grid, iters, seed, sink, st);
    default: return run<POYALGN_PEAK_MAX3_U16X2>(grid, iters, seed, sink, st);
    }
}

}  // namespace

extern "C" int poyalgn_int32_peak(int device, int kind, int iters, double* inst_per_s,
                                  float* ms, int64_t* thread_inst)
{
    using pa::set_err;
    if (kind < POYALGN_PEAK_ADD || kind > POYALGN_PEAK_MAX3_U16X2 || iters < 1 || !inst_per_s)
        return set_err(POYALGN_EINVAL, "bad peak arguments");
    int prev = -1;
    CU(cudaGetDevice(&prev));
    CU(cudaSetDevice(device));
    int nsm = 0;
    CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
    // full occupancy: 2048 threads per SM in CTAs of 256
    const int grid = nsm * 8;
    int* sink = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = 0;
    float t = 0.f;
    cudaError_t err = cudaMalloc(&sink, (size_t)grid * sizeof(int));
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    // one untimed launch brings the clocks up and loads the module
    if (err == cudaSuccess) err = launch(kind, grid, iters, 7, sink, st);
    if (err == cudaSuccess) err = cudaEventRecord(e0, st);
    if (err == cudaSuccess) err = launch(kind, grid, iters, 11, sink, st);
    if (err == cudaSuccess) err = cudaEventRecord(e1, st);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
    if (err != cudaSuccess) rc = set_err(POYALGN_ECUDA, "peak kernel: %s", cudaGetErrorString(err));
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (sink) cudaFree(sink);
    if (prev >= 0) cudaSetDevice(prev);
    if (rc) return rc;
    const double n = (double)grid * 256 * (double)iters * ROUNDS * CHAINS;
    *inst_per_s = n / (t * 1e-3);
    if (ms) *ms = t;
    if (thread_inst) *thread_inst = (int64_t)n;
    return 0;
}
