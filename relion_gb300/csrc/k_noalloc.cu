// k_noalloc.cu -- significance threshold search that allocates no memory.
//
// Some callers cannot call cudaMalloc at the point where they need this
// search: code running inside a region that must not allocate (for example
// a host thread holding a pool-allocator lock, a plugin that is only handed
// device pointers by its host application, or a caller that has budgeted all
// device memory up front).  This entry point serves them: the caller passes
// the weights and the two output arrays, and the working memory (histograms
// and per-particle state of the search) lives in one file-scope device array
// of fixed size, below.
//
// Limits and sharing rules:
//   * at most kNoAllocMaxParticles rows per call (larger calls are rejected
//     with GBR_ERR_INVALID and a message);
//   * every GPU that loads the library holds the array (about 4.3 MB) until
//     the process exits;
//   * all calls share the array and it keeps the previous call's contents:
//     each call clears what must start at zero, and calls whose work overlaps
//     on the GPU (different streams, or different host threads, without
//     ordering between them) race on it and give wrong results;
//   * the first call on each device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; with lazy module
//     loading (the CUDA default) that lookup, or the first kernel launch,
//     loads the library's device code, which may itself allocate device
//     memory.  Make the first call on each device before any stream capture
//     and outside any region that must not allocate; the guarantee holds for
//     every call after it;
//   * a row without a positive weight gets nr_significant 0 and threshold
//     +inf (gbr_expect_batch reports such a particle as "zero sum of
//     weights").
#include "../../include/gbrelion.h"
#include "gbr_internal.h"

#include <mutex>
#include <string>

namespace gbr {

constexpr int kNoAllocMaxParticles = 64;
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocScratch {
    HistBin hist[kNoAllocMaxParticles][kHistBins];
    ParticleState ps[kNoAllocMaxParticles];
    long long seg[kNoAllocMaxParticles + 1];
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

namespace {

std::mutex g_noalloc_mutex;
NoAllocScratch *g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Zero the histograms, reset the per-particle state and the row segments.
__global__ void k_noalloc_reset(NoAllocScratch *s, int n, long long len) {
    const int p = blockIdx.x;
    for (int i = threadIdx.x; i < kHistBins; i += blockDim.x) {
        s->hist[p][i].sum = 0.;
        s->hist[p][i].count = 0u;
    }
    if (threadIdx.x == 0) {
        ParticleState z{};
        z.min_coarse = 0xFFFFFFFFu;
        z.min_fine = 0xFFFFFFFFu;
        s->ps[p] = z;
        s->seg[p] = (long long)p * len;
        if (p == n - 1) s->seg[n] = (long long)n * len;
    }
}

// FP64 sum and level-0 histogram (top 12 bits) of the positive weights;
// 48 KB of dynamic shared memory (the default per-block limit).
constexpr int kChunkNA = 8192;
__global__ void k_noalloc_hist0(const float *__restrict__ w, long long len, NoAllocScratch *s) {
    extern __shared__ double na_sm[];
    double *hsum = na_sm;                                                   // [kHistBins]
    unsigned int *hcnt = reinterpret_cast<unsigned int *>(hsum + kHistBins);  // [kHistBins]
    const int p = blockIdx.y;
    const long long beg = (long long)blockIdx.x * kChunkNA;
    if (beg >= len) return;
    const long long end = min(beg + (long long)kChunkNA, len);
    for (int i = threadIdx.x; i < kHistBins; i += blockDim.x) {
        hsum[i] = 0.;
        hcnt[i] = 0u;
    }
    __syncthreads();
    const float *row = w + (size_t)p * len;
    double acc = 0.;
    for (long long e = beg + threadIdx.x; e < end; e += blockDim.x) {
        const float v = row[e];
        if (v > 0.f) {
            acc += (double)v;
            const unsigned int bin = __float_as_uint(v) >> 19;
            atomicAdd(&hsum[bin], (double)v);
            atomicAdd(&hcnt[bin], 1u);
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc != 0.) atomicAdd(&s->ps[p].sum_coarse, acc);
    __syncthreads();
    for (int i = threadIdx.x; i < kHistBins; i += blockDim.x)
        if (hcnt[i]) {
            atomicAdd(&s->hist[p][i].sum, hsum[i]);
            atomicAdd(&s->hist[p][i].count, hcnt[i]);
        }
}

// A row without a positive weight has no threshold: nr_significant 0 and
// threshold +inf (no weight passes w >= threshold).
__global__ void k_noalloc_out(const NoAllocScratch *s, int n, float *thr, unsigned int *nsig) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) {
        const bool any = s->ps[p].sum_coarse > 0.;
        thr[p] = any ? s->ps[p].thr_coarse : __int_as_float(0x7f800000);
        nsig[p] = any ? s->ps[p].nr_sign : 0u;
    }
}

int na_fail(int st, const std::string &m) {
    set_error_text(m);  // reported by gbr_last_error()
    return st;
}

}  // namespace
}  // namespace gbr

extern "C" int gbr_significance_threshold_noalloc(const float *weights, int64_t n, int64_t len,
                                                  double adaptive_fraction, float *threshold,
                                                  uint32_t *nr_significant, void *stream) {
    using namespace gbr;
    if (!weights || !threshold || !nr_significant || n <= 0 || len <= 0)
        return na_fail(GBR_ERR_INVALID, "gbr_significance_threshold_noalloc: null pointer or empty input");
    if (n > kNoAllocMaxParticles)
        return na_fail(GBR_ERR_INVALID, "gbr_significance_threshold_noalloc: " + std::to_string(n) +
                                            " rows exceed the fixed scratch of " +
                                            std::to_string(kNoAllocMaxParticles) + " rows");
    if (len > 0x7fffffffLL * (long long)kChunkNA)
        return na_fail(GBR_ERR_INVALID, "gbr_significance_threshold_noalloc: row too long");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices)
        return na_fail(GBR_ERR_CUDA, "gbr_significance_threshold_noalloc: no current CUDA device");
    NoAllocScratch *s = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess)
                return na_fail(GBR_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_noalloc_ptr[dev] = static_cast<NoAllocScratch *>(p);
        }
        s = g_noalloc_ptr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int ni = (int)n;
    k_noalloc_reset<<<ni, 256, 0, st>>>(s, ni, (long long)len);
    dim3 grid((unsigned)((len + kChunkNA - 1) / kChunkNA), ni);
    k_noalloc_hist0<<<grid, 512, kHistBins * (sizeof(double) + sizeof(unsigned int)), st>>>(weights, (long long)len, s);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = launch_select(ni, 0, adaptive_fraction, 1, s->ps, &s->hist[0][0], st);
    if (e == cudaSuccess) e = launch_hist_refine(weights, s->seg, ni, (long long)len, 1, s->ps, &s->hist[0][0], st);
    if (e == cudaSuccess) e = launch_select(ni, 1, adaptive_fraction, 1, s->ps, &s->hist[0][0], st);
    if (e == cudaSuccess) e = launch_hist_refine(weights, s->seg, ni, (long long)len, 2, s->ps, &s->hist[0][0], st);
    if (e == cudaSuccess) e = launch_select(ni, 2, adaptive_fraction, 1, s->ps, &s->hist[0][0], st);
    if (e == cudaSuccess) {
        k_noalloc_out<<<(ni + 63) / 64, 64, 0, st>>>(s, ni, threshold, nr_significant);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess)
        return na_fail(GBR_ERR_CUDA, std::string("gbr_significance_threshold_noalloc: ") + cudaGetErrorString(e));
    return GBR_OK;
}
