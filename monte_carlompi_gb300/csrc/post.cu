// Post-processing of per-photon records on the device: the reference's BRF and
// albedo arithmetic (post_processing.py:46-100 brf, :102-146 polar BRFs,
// :250-312 spectral albedo; monte_carlo3D.py:1659-1671 calculate_albedo) over
// records already in device memory, instead of re-reading the CSV text.
//
// Per config: the condition-1 exit zenith histogram weighted by wvn with
// np.histogram's binning of [0, pi/2] (edges i * (pi/2)/n, last edge pi/2;
// index ((x - 0) / (pi/2)) * n truncated, then moved one bin down when x is
// below its lower edge and one bin up when x reaches its upper edge, the last bin
// closed), wvn sums per end condition (fixed point 2^-32, so sums do not depend
// on order), counts, and sums of n_scat, path length and wavelength for the
// means the reference prints.
#include <cuda_runtime.h>

#include "mcw_internal.cuh"

namespace mcw {

namespace {

__device__ __forceinline__ int np_bin(double x, int n, double step) {
    const double last = kPi / 2;
    if (!(x >= 0.0) || !(x <= last)) return -1;
    int i = (int)((x / last) * (double)n);
    if (i == n) i -= 1;
    const double lo = (double)i * step;
    const double hi = (i + 1 == n) ? last : (double)(i + 1) * step;
    if (x < lo) i -= 1;
    else if (x >= hi && i != n - 1) i += 1;
    return i;
}

// recs: records of stride bytes whose leading fields are an mcw_record64 (kF64) or an
// mcw_record32 (the polarised records extend them).
template <bool kF64>
__global__ void post_kernel(const void *recs, size_t stride, int64_t n, int n_cfg, int n_bins, double step,
                            unsigned long long *bins_fx, unsigned int *bins_cnt, mcw_post_stats *stats) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int cond, nscat;
        uint32_t cfg;
        double wvn, theta, path;
        if (kF64) {
            const mcw_record64 r = *reinterpret_cast<const mcw_record64 *>(static_cast<const char *>(recs) + i * stride);
            cond = r.condition; nscat = r.n_scat; cfg = r.config;
            wvn = r.wvn; theta = r.theta_n; path = r.path_length;
        } else {
            const mcw_record32 r = *reinterpret_cast<const mcw_record32 *>(static_cast<const char *>(recs) + i * stride);
            cond = r.condition; nscat = r.n_scat; cfg = r.config;
            wvn = r.wvn; theta = r.theta_n; path = r.path_length;
        }
        if (cond < 1 || cond > 5 || cfg >= (uint32_t)n_cfg) continue;
        const unsigned long long wfx = (unsigned long long)llrint(wvn * 4294967296.0);
        mcw_post_stats *st = stats + cfg;
        atomicAdd(reinterpret_cast<unsigned long long *>(&st->q_cond_fx[cond]), wfx);
        atomicAdd(reinterpret_cast<unsigned long long *>(&st->n_cond[cond]), 1ull);
        atomicAdd(reinterpret_cast<unsigned long long *>(&st->sum_n_scat), (unsigned long long)nscat);
        atomicAdd(&st->sum_path_length, path);
        atomicAdd(&st->sum_wavelength, 1.0 / wvn);
        if (cond == 1 && n_bins > 0) {
            const int b = np_bin(theta, n_bins, step);
            if (b >= 0) {
                atomicAdd(bins_fx + (size_t)cfg * n_bins + b, wfx);
                atomicAdd(bins_cnt + (size_t)cfg * n_bins + b, 1u);
            }
        }
    }
}

}  // namespace

cudaError_t launch_post(const void *recs, bool f64, size_t stride, int64_t n, int n_cfg, int n_bins,
                        unsigned long long *bins_fx, unsigned int *bins_cnt, mcw_post_stats *stats, int sms,
                        cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const double step = (kPi / 2) / (double)(n_bins > 0 ? n_bins : 1);
    const int64_t want = (n + 255) / 256;
    const int grid = (int)(want < (int64_t)sms * 8 ? want : (int64_t)sms * 8);
    if (f64) post_kernel<true><<<grid, 256, 0, s>>>(recs, stride, n, n_cfg, n_bins, step, bins_fx, bins_cnt, stats);
    else post_kernel<false><<<grid, 256, 0, s>>>(recs, stride, n, n_cfg, n_bins, step, bins_fx, bins_cnt, stats);
    return cudaGetLastError();
}

}  // namespace mcw
