// Shot sampling from outcome probabilities on the device (no reference counterpart:
// the reference backend reports probabilities only, max_shots = 1).
//
// The 2**m probabilities are turned into a cumulative distribution by a
// two-level scan (1024-value blocks in shared memory, then the block
// totals); every shot draws a counter-based uniform (splitmix64 of the seed
// and the shot index), finds its outcome by binary search in the CDF and
// increments that outcome's count.  Negative probabilities (rounding noise
// of a measurement) count as zero; when no probability is positive no shot
// is drawn and every count stays 0.
#include "dm_common.cuh"

namespace dmg {
namespace sample {

constexpr int kScanThreads = 256;
constexpr int kScanBlock = 4 * kScanThreads;   // values per scan block
constexpr int kMaxBits = 20;

// splitmix64 (S. Vigna): a 64-bit mixing function of a counter.
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// inclusive scan of max(p, 0) inside each block of kScanBlock values; block totals to sums
__global__ void __launch_bounds__(kScanThreads) scan_blocks(const double *__restrict__ p, int64_t count,
                                                            double *__restrict__ cdf, double *__restrict__ sums) {
    __shared__ double s[kScanBlock];
    const int64_t base = int64_t(blockIdx.x) * kScanBlock;
    for (int i = threadIdx.x; i < kScanBlock; i += kScanThreads) {
        const int64_t g = base + i;
        s[i] = g < count ? fmax(p[g], 0.0) : 0.0;
    }
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {     // Hillis-Steele over the block
        double add[4];
        for (int k = 0; k < 4; ++k) {
            const int i = threadIdx.x + k * kScanThreads;
            add[k] = i >= off ? s[i - off] : 0.0;
        }
        __syncthreads();
        for (int k = 0; k < 4; ++k) s[threadIdx.x + k * kScanThreads] += add[k];
        __syncthreads();
    }
    for (int i = threadIdx.x; i < kScanBlock; i += kScanThreads) {
        const int64_t g = base + i;
        if (g < count) cdf[g] = s[i];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = s[kScanBlock - 1];
}

// exclusive scan of the block totals (one thread: at most 1024 blocks), then offsets added
__global__ void scan_sums(double *__restrict__ sums, int nblocks) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double run = 0.0;
        for (int b = 0; b < nblocks; ++b) {
            const double v = sums[b];
            sums[b] = run;
            run += v;
        }
        sums[nblocks] = run;
    }
}

__global__ void add_offsets(double *__restrict__ cdf, int64_t count, const double *__restrict__ sums) {
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < count; g += int64_t(gridDim.x) * blockDim.x)
        cdf[g] += sums[g / kScanBlock];
}

__global__ void draw(const double *__restrict__ cdf, int64_t count, const double *__restrict__ total, int64_t shots,
                     uint64_t seed, unsigned long long *__restrict__ counts) {
    const double tot = *total;
    if (!(tot > 0.0)) return;   // nothing to draw from: the counts stay 0 (the caller sees their sum)
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < shots; i += int64_t(gridDim.x) * blockDim.x) {
        const uint64_t r = splitmix64(seed ^ splitmix64(uint64_t(i)));
        const double u = double(r >> 11) * (1.0 / 9007199254740992.0) * tot;   // [0, tot)
        int64_t lo = 0, hi = count - 1;                  // first k with cdf[k] > u
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (cdf[mid] > u) hi = mid;
            else lo = mid + 1;
        }
        atomicAdd(counts + lo, 1ull);
    }
}

}  // namespace sample
}  // namespace dmg

using namespace dmg;

extern "C" size_t dm_sample_counts_scratch_bytes(int m) {
    if (m < 1 || m > sample::kMaxBits) return 0;
    const int64_t count = int64_t(1) << m;
    const int64_t nb = (count + sample::kScanBlock - 1) / sample::kScanBlock;
    return size_t(count + nb + 1) * sizeof(double);
}

extern "C" int dm_sample_counts(const double *probs_dev, int m, int64_t shots, uint64_t seed, int64_t *counts_dev,
                                void *scratch_dev, void *stream) {
    DM_CHECK_ARG(probs_dev && counts_dev && scratch_dev && m >= 1 && m <= sample::kMaxBits && shots >= 0);
    const int64_t count = int64_t(1) << m;
    const int nb = int((count + sample::kScanBlock - 1) / sample::kScanBlock);
    double *cdf = static_cast<double *>(scratch_dev);
    double *sums = cdf + count;
    cudaStream_t s = as_stream(stream);
    DM_CUDA_TRY(cudaMemsetAsync(counts_dev, 0, size_t(count) * sizeof(int64_t), s));
    sample::scan_blocks<<<nb, sample::kScanThreads, 0, s>>>(probs_dev, count, cdf, sums);
    sample::scan_sums<<<1, 32, 0, s>>>(sums, nb);
    sample::add_offsets<<<grid_for(count, 256), 256, 0, s>>>(cdf, count, sums);
    count_launch(3);
    if (shots > 0) {
        sample::draw<<<grid_for(shots, 256), 256, 0, s>>>(cdf, count, sums + nb, shots, seed,
                                                           reinterpret_cast<unsigned long long *>(counts_dev));
        count_launch();
    }
    return launch_status();
}
