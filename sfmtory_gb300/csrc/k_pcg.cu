// Vector side of the matrix-free Schur-complement PCG (image level: a free
// camera of one image is part of that image's block; a camera shared by
// several images is one slot block kept as copies in its images' blocks, see
// k_shared.cu):
//
//   S p = (H + lambda diag H) p - sum_p E_p^T C_p^-1 E_p p
//
// The observation passes that apply S and build the block-Jacobi
// preconditioner live in k_matfree.cu; this file sums the image pass's
// partials into q, runs the CG recurrences and scatters the solution.
// Scalars of the iteration live in the device state so the host only polls
// for convergence every few iterations. Vectors are in the kernel precision
// (FP32 on the mixed path); every dot product accumulates in FP64.
#include <type_traits>

#include "kernels.cuh"

namespace sfmba {

namespace {

template <typename T>
__device__ __forceinline__ void kahan_add(T &s, T &c, T x) {
    if constexpr (std::is_same<T, float>::value) {
        const T y = x - c;
        const T t = s + y;
        c = (t - s) - y;
        s = t;
    } else {
        s += x;
    }
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// v[t] + v[t + B] + v[t + 2B] + ... for thread t of a B-thread block, added
// in that order, with the loads issued eight at a time (the sums are L2
// round trips otherwise serialised by the add chain).
__device__ __forceinline__ double strided_sum(const double *__restrict__ v, int n) {
    const int B = blockDim.x;
    double a = 0.0;
    int k = threadIdx.x;
    for (; k + 7 * B < n; k += 8 * B) {
        double w[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) w[u] = v[k + u * B];
#pragma unroll
        for (int u = 0; u < 8; ++u) a += w[u];
    }
    for (; k < n; k += B) a += v[k];
    return a;
}

__global__ void k_pcg_scalar_init(const double *part, int nI, double tol2, LMState *st) {
    __shared__ double sh[256];
    double a = strided_sum(part, nI), b = strided_sum(part + nI, nI);
    a = block_sum(a, sh);
    b = block_sum(b, sh);
    if (threadIdx.x == 0) {
        st->pcg_rzbuf[0] = a;
        st->pcg_rzbuf[1] = 0.0;
        st->pcg_bb = b;
        st->pcg_rr = b;
        st->pcg_tol2 = tol2;
        st->pcg_iterations = 0;
        st->pcg_done = (b > 0.0 && a > 0.0 && isfinite(a)) ? 0 : 1;
        st->pcg_alpha = 0.0;
        st->pcg_beta = 0.0;
    }
}

// q_i = (H_i + lambda diag H_i) p_i - sum of the image's partials; part[i] =
// p_i . q_i over the image's own columns (pmask; a shared camera's columns
// are added by launch_shared_qreduce once summed over its images).
template <typename T, int D>
__global__ void __launch_bounds__(128) k_pcg_images_finish(const T *__restrict__ ipart,
                                                           const int *__restrict__ ipart_off,
                                                           const double *__restrict__ img_H,
                                                           const int *__restrict__ img_active,
                                                           const int *__restrict__ img_pmask,
                                                           const T *__restrict__ p, const LMState *__restrict__ st,
                                                           int nI, T *__restrict__ q, double *__restrict__ part) {
    if (st->pcg_done) return;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nI) return;
    const double lam = st->lambda;
    const int act = img_active[i];
    const int pm = img_pmask[i];
    const double *H = img_H + (size_t)i * D * D;
    const T *pv = p + (size_t)i * D;
    double pq = 0.0;
    if (lane < D) {
        const int c = lane;
        double sch = 0.0;
        const int k1 = ipart_off[i + 1];
        int k = ipart_off[i];
        for (; k + 8 <= k1; k += 8) {  // loads eight at a time, added in chunk order
            T w[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) w[u] = ipart[(size_t)(k + u) * D + c];
#pragma unroll
            for (int u = 0; u < 8; ++u) sch += (double)w[u];
        }
        for (; k < k1; ++k) sch += (double)ipart[(size_t)k * D + c];
        double hp = 0.0;
#pragma unroll
        for (int d = 0; d < D; ++d) hp += H[c * D + d] * (double)pv[d];
        hp += lam * H[c * D + c] * (double)pv[c];
        const double qc = ((act >> c) & 1) ? hp - sch : 0.0;
        q[(size_t)i * D + c] = (T)qc;
        if ((pm >> c) & 1) pq = (double)pv[c] * (double)(T)qc;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) pq += __shfl_xor_sync(0xffffffffu, pq, off);
    if (lane == 0) part[2 * nI + i] = pq;
}

__global__ void k_point_chunks(const int *pt_start, int nP, long long nO, int nchunks, int *pchunk) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > nchunks) return;
    long long t = (long long)k * kChunkObs;
    if (t > nO) t = nO;
    int lo = 0, hi = nP;  // first point whose start is >= t (pt_start[nP] == nO)
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (pt_start[mid] < t) lo = mid + 1;
        else hi = mid;
    }
    pchunk[k] = k == nchunks ? (int)nO : pt_start[lo];
}


// x += alpha p; r -= alpha q; z = M^-1 r; per-image partials of r.z and
// r.r over the columns dmask counts. alpha = (r.z) / (p.q) with p.q reduced
// from the image pass's partials by every block in the same order (no
// separate scalar kernel). One warp per image, 8 images per block.
template <typename T, int D>
__global__ void __launch_bounds__(256) k_pcg_update(const T *Minv, const T *p, const T *q, const int *img_dmask,
                                                    LMState *st, int nI, int parity, T *x, T *r, T *z,
                                                    double *part) {
    __shared__ double sh[256];
    if (st->pcg_done) return;
    double a = strided_sum(part + 2 * nI, nI);
    a = block_sum(a, sh);
    if (!(a > 0.0) || !isfinite(a)) {  // breakdown: keep the current iterate
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            st->pcg_done = 1;
            st->pcg_breakdowns += 1;
            st->pcg_alpha = 0.0;
        }
        return;
    }
    const double alpha = st->pcg_rzbuf[parity] / a;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->pcg_alpha = alpha;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nI) return;
    const size_t base = (size_t)i * D;
    T rc = T(0);
    if (lane < D) {
        x[base + lane] = (T)((double)x[base + lane] + alpha * (double)p[base + lane]);
        rc = (T)((double)r[base + lane] - alpha * (double)q[base + lane]);
        r[base + lane] = rc;
    }
    double zc = 0.0;
    const T *M = Minv + (size_t)i * D * D;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const T rd = __shfl_sync(0xffffffffu, rc, d);
        if (lane < D) zc += (double)M[lane * D + d] * (double)rd;
    }
    double rz = 0.0, rr = 0.0;
    if (lane < D) {
        z[base + lane] = (T)zc;
        if ((img_dmask[i] >> lane) & 1) {
            rz = (double)rc * (double)(T)zc;
            rr = (double)rc * (double)rc;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        rz += __shfl_xor_sync(0xffffffffu, rz, off);
        rr += __shfl_xor_sync(0xffffffffu, rr, off);
    }
    if (lane == 0) {
        part[i] = rz;
        part[nI + i] = rr;
    }
}

// Convergence test and p = z + beta p, beta = (r.z)_new / (r.z)_old. Every
// block reduces the partials itself; block 0 records the new r.z in the
// other parity slot (read by the next iteration only) and the counters.
// img_owner (shared cameras, else NULL): a linked image's camera entries of
// z are its owner's, so p stays a copy of the owner's there.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_dir(const T *z, LMState *st, const double *part, int nI, int nID,
                                                 int parity, T *p, int D, T *p4, const int *img_owner) {
    __shared__ double sh[256];
    if (st->pcg_done) return;
    double a = strided_sum(part, nI), b = strided_sum(part + nI, nI);
    a = block_sum(a, sh);
    b = block_sum(b, sh);
    const bool stop = b <= st->pcg_tol2 * st->pcg_bb || !(a > 0.0) || !isfinite(a);
    const double beta = stop ? 0.0 : a / st->pcg_rzbuf[parity];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->pcg_iterations += 1;
        st->pcg_total += 1;
        st->pcg_rr = b;
        if (stop) {
            st->pcg_done = 1;
            if (!(b <= st->pcg_tol2 * st->pcg_bb)) st->pcg_breakdowns += 1;
        } else {
            st->pcg_beta = beta;
            st->pcg_rzbuf[parity ^ 1] = a;
        }
    }
    if (stop) return;
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nID) return;
    int zu = u;
    if (img_owner) {
        const int i = u / D, c = u - i * D;
        if (c >= 6) zu = img_owner[i] * D + c;
    }
    const T pn = (T)((double)z[zu] + beta * (double)p[u]);
    p[u] = pn;
    if (p4) {
        const int i = u / D;
        store_dir(reinterpret_cast<float *>(p4), nI, i, u - i * D, (float)pn);
    }
}

template <typename T>
__global__ void k_pcg_scatter(const T *x, const int *pre_start, const int *pre, const unsigned char *masked,
                              int n, double *delta) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    double v = 0.0;
    if (!masked[a] && pre_start[a] < pre_start[a + 1]) v = (double)x[pre[pre_start[a]]];
    delta[a] = v;
}

template <typename F>
void dispatch_D(int D, F &&f) {
    switch (D) {
    case 6: f(std::integral_constant<int, 6>()); break;
    case 9: f(std::integral_constant<int, 9>()); break;
    case 10: f(std::integral_constant<int, 10>()); break;
    case 11: f(std::integral_constant<int, 11>()); break;
    case 14: f(std::integral_constant<int, 14>()); break;
    default: throw Error(SFMBA_ERR_INTERNAL, "unsupported image block width");
    }
}

template <typename T, int D>
void images_finish_t(const Bufs &b, cudaStream_t s) {
    k_pcg_images_finish<T, D><<<div_up(b.nI, 4), 128, 0, s>>>((const T *)b.ipart, b.ipart_off, b.img_H,
                                                              b.img_active, b.img_pmask, (const T *)b.pcg_p, b.state,
                                                              b.nI, (T *)b.pcg_q, b.pcg_part);
    SFMBA_LAUNCH_CHECK();
    if (b.sh.nsh > 0) launch_shared_qreduce(b, s);
}

template <typename T, int D>
void vector_t(const Bufs &b, cudaStream_t s, int parity, bool coarse) {
    k_pcg_update<T, D><<<div_up(b.nI, 8), 256, 0, s>>>((const T *)b.pcg_Minv, (const T *)b.pcg_p,
                                                       (const T *)b.pcg_q, b.img_dmask, b.state, b.nI, parity,
                                                       (T *)b.pcg_x, (T *)b.pcg_r, (T *)b.pcg_z, b.pcg_part);
    SFMBA_LAUNCH_CHECK();
    if (coarse) launch_coarse_correct(b, false, s);  // z += Z A_c^-1 Z^T r, new r.z partials
    k_pcg_dir<T><<<div_up(b.nID, 256), 256, 0, s>>>((const T *)b.pcg_z, b.state, b.pcg_part, b.nI, b.nID, parity,
                                                    (T *)b.pcg_p, b.D,
                                                    std::is_same<T, float>::value ? (T *)(void *)b.pcg_p4 : nullptr,
                                                    b.sh.nsh > 0 ? b.sh.img_owner : nullptr);
    SFMBA_LAUNCH_CHECK();
}

}  // namespace

void launch_pcg_start(const Bufs &b, cudaStream_t s) {
    k_pcg_scalar_init<<<1, 256, 0, s>>>(b.pcg_part, b.nI, b.pcg_tol * b.pcg_tol, b.state);
    SFMBA_LAUNCH_CHECK();
}

#define SFMBA_PCG_LAUNCHER(name, impl)                           \
    void name(const Bufs &b, cudaStream_t s) {                   \
        dispatch_D(b.D, [&](auto dc) {                           \
            constexpr int D = decltype(dc)::value;               \
            if (b.mixed) impl<float, D>(b, s);                   \
            else impl<double, D>(b, s);                          \
        });                                                      \
    }
SFMBA_PCG_LAUNCHER(launch_pcg_images_finish, images_finish_t)
#undef SFMBA_PCG_LAUNCHER

void launch_pcg_vector(const Bufs &b, cudaStream_t s, int parity, bool coarse) {
    dispatch_D(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        if (b.mixed) vector_t<float, D>(b, s, parity, coarse);
        else vector_t<double, D>(b, s, parity, coarse);
    });
}

void launch_pcg_partition(Bufs &b, cudaStream_t s) {
    b.npchunks = (int)((b.nO + kChunkObs - 1) / kChunkObs);
    k_point_chunks<<<div_up(b.npchunks + 1, 256), 256, 0, s>>>(b.pt_start, b.nP, b.nO, b.npchunks, b.pchunk);
    SFMBA_LAUNCH_CHECK();
}

void launch_pcg_finish(const Bufs &b, double *delta_slot, cudaStream_t s) {
    if (b.n == 0) return;
    if (b.mixed)
        k_pcg_scatter<float><<<div_up(b.n, 256), 256, 0, s>>>((const float *)b.pcg_x, b.slot_pre_start,
                                                              b.slot_pre, b.slot_masked, b.n, delta_slot);
    else
        k_pcg_scatter<double><<<div_up(b.n, 256), 256, 0, s>>>((const double *)b.pcg_x, b.slot_pre_start,
                                                               b.slot_pre, b.slot_masked, b.n, delta_slot);
    SFMBA_LAUNCH_CHECK();
}

}  // namespace sfmba
