// Problem set-up on the device: validation, visibility sort of the
// observations (point-major, and an image-major permutation of it) and the
// image-pair list the Schur reduction walks.
#include <cub/cub.cuh>

#include "kernels.cuh"

namespace sfmba {

namespace {

__global__ void k_validate(const int *cam_of_img, const int *cam_model, const int *obs_image,
                           const int *obs_point, long long nO, int nI, int nC, int nP, int *bad) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < nO) {
        int i = obs_image[t], p = obs_point[t];
        if (i < 0 || i >= nI || p < 0 || p >= nP) atomicOr(bad, 1);
    }
    if (t < nI) {
        int c = cam_of_img[t];
        if (c < 0 || c >= nC) atomicOr(bad, 2);
    }
    if (t < nC) {
        int m = cam_model[t];
        if (m < 0 || m > 5) atomicOr(bad, 4);
    }
}

__global__ void k_iota(int *v, long long n) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n) v[t] = (int)t;
}

__global__ void k_gather_obs(const int *sorted_pt, const int *perm, const int *obs_image_in,
                             const double *obs_xy_in, long long nO, int *ob_pt, int *ob_img,
                             double2 *ob_xy, int *img_keys) {
    long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (o >= nO) return;
    int src = perm[o];
    ob_pt[o] = sorted_pt[o];
    int i = obs_image_in[src];
    ob_img[o] = i;
    img_keys[o] = i;
    ob_xy[o] = make_double2(obs_xy_in[2 * (long long)src], obs_xy_in[2 * (long long)src + 1]);
}

// start[k] = first index whose sorted key is >= k, for k in [0, nk].
__global__ void k_segment_starts(const int *sorted_keys, long long n, int nk, int *start) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > nk) return;
    long long lo = 0, hi = n;
    while (lo < hi) {
        long long mid = (lo + hi) >> 1;
        if (sorted_keys[mid] < k) lo = mid + 1;
        else hi = mid;
    }
    start[k] = (int)lo;
}

// Ordered observation pairs (a, b) of one point with image(a) <= image(b):
// every block product of the point's Schur term is one such pair, the pair
// (b, a) of an image pair i < j being recovered by transposition.
__global__ void k_count_pairs(const int *pt_start, const int *ob_img, int nP, long long *count) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nP) return;
    int s = pt_start[p], e = pt_start[p + 1];
    long long c = 0;
    for (int a = s; a < e; ++a) {
        int ia = ob_img[a];
        for (int b = s; b < e; ++b) c += (ia <= ob_img[b]) ? 1 : 0;
    }
    count[p] = c;
}

__global__ void k_emit_pairs(const int *pt_start, const int *ob_img, int nP, int nI,
                             const long long *incl_scan, unsigned *keys, int2 *vals) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nP) return;
    int s = pt_start[p], e = pt_start[p + 1];
    long long off = p == 0 ? 0 : incl_scan[p - 1];
    for (int a = s; a < e; ++a) {
        int ia = ob_img[a];
        for (int b = s; b < e; ++b) {
            int ib = ob_img[b];
            if (ia <= ib) {
                keys[off] = (unsigned)ia * (unsigned)nI + (unsigned)ib;
                vals[off] = make_int2(a, b);
                ++off;
            }
        }
    }
}

__global__ void k_iota(int *v, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

__global__ void k_group_decode(const unsigned *unique_keys, const int *d_ngroups, int nI,
                               int2 *group_ij) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= *d_ngroups) return;
    unsigned k = unique_keys[g];
    group_ij[g] = make_int2((int)(k / (unsigned)nI), (int)(k % (unsigned)nI));
}

__global__ void k_fill(int *a, long long n, int v) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n) a[t] = v;
}

__global__ void k_min_image(const int *obs_point, const int *obs_image, long long nO, int *key) {
    const long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (o < nO) atomicMin(key + obs_point[o], obs_image[o]);
}

__global__ void k_invert(const int *perm, int n, int *inv) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) inv[perm[k]] = k;
}

__global__ void k_remap(const int *in, const int *map, long long n, int *out) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n) out[t] = map[in[t]];
}

__global__ void k_gather_points(const double *src, const int *perm, int nP, double *dst) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nP) return;
    const int o = perm[k];
    dst[3 * (size_t)k] = src[3 * (size_t)o];
    dst[3 * (size_t)k + 1] = src[3 * (size_t)o + 1];
    dst[3 * (size_t)k + 2] = src[3 * (size_t)o + 2];
}

__global__ void k_scatter_points(const double *src, const int *old2new, int nP, double *dst) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nP) return;
    const int k = old2new[o];
    dst[3 * (size_t)o] = src[3 * (size_t)k];
    dst[3 * (size_t)o + 1] = src[3 * (size_t)k + 1];
    dst[3 * (size_t)o + 2] = src[3 * (size_t)k + 2];
}

int bits_for(long long v) {
    int b = 1;
    while ((1LL << b) <= v) ++b;
    return b;
}

}  // namespace

void validate_problem_device(const int *cam_of_img, const int *cam_model, const int *obs_image,
                             const int *obs_point, long long nO, int nI, int nC, int nP,
                             int *d_bad, cudaStream_t s) {
    long long n = nO;
    if (nI > n) n = nI;
    if (nC > n) n = nC;
    if (n == 0) return;
    k_validate<<<div_up(n, 256), 256, 0, s>>>(cam_of_img, cam_model, obs_image, obs_point, nO, nI,
                                              nC, nP, d_bad);
    SFMBA_LAUNCH_CHECK();
}

size_t sort_temp_bytes(long long nO, int nP, int nI) {
    size_t a = 0, b = 0, c = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, a, (int *)nullptr, (int *)nullptr, (int *)nullptr,
                                    (int *)nullptr, (int)nO, 0, bits_for(nP));
    cub::DeviceRadixSort::SortPairs(nullptr, b, (int *)nullptr, (int *)nullptr, (int *)nullptr,
                                    (int *)nullptr, (int)nO, 0, bits_for(nI));
    cub::DeviceRadixSort::SortPairs(nullptr, c, (int *)nullptr, (int *)nullptr, (int *)nullptr,
                                    (int *)nullptr, nP, 0, bits_for((long long)nI + 1));
    size_t m = a > b ? a : b;
    return m > c ? m : c;
}

void order_points(const int *obs_point_in, const int *obs_image_in, long long nO, int nP, int nI, int *key,
                  int *key_sorted, int *iota_tmp, int *perm, int *old2new, int *obs_point_out, void *temp,
                  size_t temp_bytes, cudaStream_t s) {
    if (nP == 0) return;
    k_fill<<<div_up(nP, 256), 256, 0, s>>>(key, nP, nI);  // points without observations go last
    SFMBA_LAUNCH_CHECK();
    if (nO > 0) {
        k_min_image<<<div_up(nO, 256), 256, 0, s>>>(obs_point_in, obs_image_in, nO, key);
        SFMBA_LAUNCH_CHECK();
    }
    k_iota<<<div_up(nP, 256), 256, 0, s>>>(iota_tmp, nP);
    SFMBA_LAUNCH_CHECK();
    size_t tb = temp_bytes;
    SFMBA_CUDA(cub::DeviceRadixSort::SortPairs(temp, tb, key, key_sorted, iota_tmp, perm, nP, 0,
                                               bits_for((long long)nI + 1), s));
    k_invert<<<div_up(nP, 256), 256, 0, s>>>(perm, nP, old2new);
    SFMBA_LAUNCH_CHECK();
    if (nO > 0) {
        k_remap<<<div_up(nO, 256), 256, 0, s>>>(obs_point_in, old2new, nO, obs_point_out);
        SFMBA_LAUNCH_CHECK();
    }
}

void gather_points(const double *src, const int *perm, int nP, double *dst, cudaStream_t s) {
    if (nP == 0) return;
    k_gather_points<<<div_up(nP, 256), 256, 0, s>>>(src, perm, nP, dst);
    SFMBA_LAUNCH_CHECK();
}

void scatter_points(const double *src, const int *old2new, int nP, double *dst, cudaStream_t s) {
    if (nP == 0) return;
    k_scatter_points<<<div_up(nP, 256), 256, 0, s>>>(src, old2new, nP, dst);
    SFMBA_LAUNCH_CHECK();
}

void sort_observations(const int *obs_point_in, const int *obs_image_in, const double *obs_xy_in,
                       long long nO, int nP, int nI, Bufs &b, void *temp, size_t temp_bytes,
                       int *keys_tmp, int *vals_tmp, int *keys_tmp2, int *vals_tmp2,
                       cudaStream_t s) {
    if (nO > 0) {
        k_iota<<<div_up(nO, 256), 256, 0, s>>>(vals_tmp, nO);
        SFMBA_LAUNCH_CHECK();
        size_t tb = temp_bytes;
        SFMBA_CUDA(cub::DeviceRadixSort::SortPairs(temp, tb, obs_point_in, keys_tmp2, vals_tmp,
                                                   vals_tmp2, (int)nO, 0, bits_for(nP), s));
        k_gather_obs<<<div_up(nO, 256), 256, 0, s>>>(keys_tmp2, vals_tmp2, obs_image_in, obs_xy_in,
                                                     nO, b.ob_pt, b.ob_img, b.ob_xy, keys_tmp);
        SFMBA_LAUNCH_CHECK();
    }
    k_segment_starts<<<div_up(nP + 1, 256), 256, 0, s>>>(b.ob_pt, nO, nP, b.pt_start);
    SFMBA_LAUNCH_CHECK();
    if (nO > 0) {
        k_iota<<<div_up(nO, 256), 256, 0, s>>>(vals_tmp, nO);
        SFMBA_LAUNCH_CHECK();
        size_t tb = temp_bytes;
        SFMBA_CUDA(cub::DeviceRadixSort::SortPairs(temp, tb, keys_tmp, keys_tmp2, vals_tmp,
                                                   b.img_obs, (int)nO, 0, bits_for(nI), s));
    }
    k_segment_starts<<<div_up(nI + 1, 256), 256, 0, s>>>(keys_tmp2, nO, nI, b.img_start);
    SFMBA_LAUNCH_CHECK();
}

size_t pairs_temp_bytes(long long npairs, int nI) {
    size_t a = 0, b = 0, c = 0, d = 0;
    int n = (int)(npairs > 0 ? npairs : 1);
    cub::DeviceRadixSort::SortPairs(nullptr, a, (unsigned *)nullptr, (unsigned *)nullptr,
                                    (int2 *)nullptr, (int2 *)nullptr, n, 0,
                                    bits_for((long long)nI * nI));
    cub::DeviceRunLengthEncode::Encode(nullptr, b, (unsigned *)nullptr, (unsigned *)nullptr,
                                       (int *)nullptr, (int *)nullptr, n);
    cub::DeviceScan::ExclusiveSum(nullptr, c, (int *)nullptr, (int *)nullptr, n + 1);
    size_t m = a;
    if (b > m) m = b;
    if (c > m) m = c;
    if (d > m) m = d;
    return m;
}

long long count_pairs(const Bufs &b, long long *d_count_scan, void *temp, size_t temp_bytes,
                      cudaStream_t s) {
    if (b.nP == 0) return 0;
    k_count_pairs<<<div_up(b.nP, 256), 256, 0, s>>>(b.pt_start, b.ob_img, b.nP, d_count_scan);
    SFMBA_LAUNCH_CHECK();
    size_t need = 0;
    SFMBA_CUDA(cub::DeviceScan::InclusiveSum(nullptr, need, d_count_scan, d_count_scan, b.nP, s));
    if (need > temp_bytes) throw Error(SFMBA_ERR_INTERNAL, "scan temp too small");
    size_t tb = temp_bytes;
    SFMBA_CUDA(cub::DeviceScan::InclusiveSum(temp, tb, d_count_scan, d_count_scan, b.nP, s));
    long long total = 0;
    SFMBA_CUDA(cudaMemcpyAsync(&total, d_count_scan + (b.nP - 1), sizeof(long long),
                               cudaMemcpyDeviceToHost, s));
    SFMBA_CUDA(cudaStreamSynchronize(s));
    return total;
}

void build_pairs(Bufs &b, const long long *d_count_scan, unsigned *keys_a, unsigned *keys_b,
                 int2 *vals_b, void *temp, size_t temp_bytes, int *d_ngroups, cudaStream_t s) {
    if (b.npairs == 0) {
        b.ngroups = 0;
        return;
    }
    k_emit_pairs<<<div_up(b.nP, 256), 256, 0, s>>>(b.pt_start, b.ob_img, b.nP, b.nI, d_count_scan,
                                                   keys_a, b.pairs);
    SFMBA_LAUNCH_CHECK();
    int np = (int)b.npairs;
    size_t tb = temp_bytes;
    SFMBA_CUDA(cub::DeviceRadixSort::SortPairs(temp, tb, keys_a, keys_b, b.pairs, vals_b, np, 0,
                                               bits_for((long long)b.nI * b.nI), s));
    SFMBA_CUDA(cudaMemcpyAsync(b.pairs, vals_b, sizeof(int2) * (size_t)np,
                               cudaMemcpyDeviceToDevice, s));
    // Unique image-pair keys and their run lengths -> group starts.
    int *counts = reinterpret_cast<int *>(vals_b);  // reuse: vals_b no longer needed
    tb = temp_bytes;
    SFMBA_CUDA(cub::DeviceRunLengthEncode::Encode(temp, tb, keys_b, keys_a, counts, d_ngroups, np, s));
    int ng = 0;
    SFMBA_CUDA(cudaMemcpyAsync(&ng, d_ngroups, sizeof(int), cudaMemcpyDeviceToHost, s));
    SFMBA_CUDA(cudaStreamSynchronize(s));
    b.ngroups = ng;
    SFMBA_CUDA(cudaMemsetAsync(counts + ng, 0, sizeof(int), s));
    tb = temp_bytes;
    SFMBA_CUDA(cub::DeviceScan::ExclusiveSum(temp, tb, counts, b.group_start, ng + 1, s));
    k_group_decode<<<div_up(ng, 256), 256, 0, s>>>(keys_a, d_ngroups, b.nI, b.group_ij);
    SFMBA_LAUNCH_CHECK();
    // Launch order of the Schur kernels: the groups with the most pairs first
    // (stable, so equal counts keep their order), so the long groups do not
    // start last and leave the GPU idle behind them.
    int *iota = counts + (np + 1);  // the upper half of vals_b
    k_iota<<<div_up(ng, 256), 256, 0, s>>>(iota, ng);
    SFMBA_LAUNCH_CHECK();
    size_t need = 0;
    SFMBA_CUDA(cub::DeviceRadixSort::SortPairsDescending(nullptr, need, counts, (int *)keys_b, iota, b.group_order, ng,
                                                         0, 32, s));
    if (need > temp_bytes) throw Error(SFMBA_ERR_INTERNAL, "group sort temp too small");
    tb = temp_bytes;
    SFMBA_CUDA(cub::DeviceRadixSort::SortPairsDescending(temp, tb, counts, (int *)keys_b, iota, b.group_order, ng, 0,
                                                         32, s));
}

}  // namespace sfmba
