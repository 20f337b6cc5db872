// Free cameras shared by several images on the matrix-free PCG solver.
//
// The reference gives a camera one slot block however many images use it
// and folds every image's camera terms onto it (crates/sfm-ba/src/lib.rs:
// 753-787 slotting, :891-908 camera blocks, :946-956 pose x camera cross
// blocks). The PCG works on image-level vectors, so the slot-level system is
// applied as S_slot = P^T S_img P, P copying a camera's slot entries into
// the camera columns of each image that uses it ("linked" images):
//   * p is kept replicated on those columns (the observation passes read an
//     image's columns as they are), and q = S p is summed over the camera's
//     images and copied back to all of them (k_sh_qreduce);
//   * damping is linear in the blocks (lambda diag of a sum = sum of lambda
//     diag), so the per-image damped blocks add up to the slot block;
//   * dot products count a camera's entries once, on its owner image (the
//     first image using it), through the PCG kernels' column masks.
// The preconditioner is block-Jacobi over slot blocks: a linked image's own
// block covers its pose columns only, and each shared camera gets its exact
// diagonal block of the reduced system,
//   A_c = sum_{i in c} (H_i + lambda diag H_i)_cc - sum_p Y_pc^T C_p^-1 Y_pc,
// Y_pc = sum over point p's observations in images of camera c of
// Jx~^T Jc~ (camera columns): one thread per point forms the point's
// Y_pc^T C_p^-1 Y_pc per (point, camera) incidence, the incidences sorted
// by camera are summed per chunk and the chunks per camera in a fixed order
// (no float atomics: reproducible).
#include <cub/cub.cuh>

#include "mf_passes.cuh"

namespace sfmba {

namespace {

// Distinct shared cameras among a point's observations.
__global__ void k_sh_count(const int *__restrict__ pt_start, const int *__restrict__ ob_img,
                           const int *__restrict__ img_shcam, int nP, long long *__restrict__ count) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > nP) return;
    if (p == nP) {
        count[nP] = 0;
        return;
    }
    const int o0 = pt_start[p], o1 = pt_start[p + 1];
    long long k = 0;
    for (int o = o0; o < o1; ++o) {
        const int sc = img_shcam[ob_img[o]];
        if (sc < 0) continue;
        bool first = true;
        for (int o2 = o0; o2 < o && first; ++o2) first = img_shcam[ob_img[o2]] != sc;
        k += first ? 1 : 0;
    }
    count[p] = k;
}

// Key (camera) and value (incidence) of every incidence, in point order and,
// within a point, in order of the camera's first observation.
__global__ void k_sh_emit(const int *__restrict__ pt_start, const int *__restrict__ ob_img,
                          const int *__restrict__ img_shcam, const long long *__restrict__ inc_off, int nP,
                          int *__restrict__ key, int *__restrict__ val) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nP) return;
    const int o0 = pt_start[p], o1 = pt_start[p + 1];
    long long slot = inc_off[p];
    for (int o = o0; o < o1; ++o) {
        const int sc = img_shcam[ob_img[o]];
        if (sc < 0) continue;
        bool first = true;
        for (int o2 = o0; o2 < o && first; ++o2) first = img_shcam[ob_img[o2]] != sc;
        if (!first) continue;
        key[slot] = sc;
        val[slot] = (int)slot;
        ++slot;
    }
}

__global__ void k_sh_key_counts(const int *__restrict__ key, long long n, int *__restrict__ counts) {
    // The keys are sorted: a run's first and last elements add their bounds.
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int k = key[t];
    const bool first = t == 0 || key[t - 1] != k;
    const bool last = t == n - 1 || key[t + 1] != k;
    if (first && last) atomicAdd(&counts[k], 1);
    else if (first) atomicAdd(&counts[k], -(int)t);
    else if (last) atomicAdd(&counts[k], (int)(t + 1));
}

// Upper triangle of Y_pc^T C_p^-1 Y_pc for each incidence of point p, in the
// incidence order of k_sh_emit. A point without a usable inverse
// contributes nothing (its Schur terms are skipped everywhere, lib.rs:964).
template <typename T, int D, bool RC, int M>
__global__ void __launch_bounds__(128) k_sh_inc(JacSrc<T> J, const int *__restrict__ pt_start,
                                                const int *__restrict__ img_shcam,
                                                const long long *__restrict__ inc_off, int nP,
                                                const T *__restrict__ pt_Cinv, const unsigned char *__restrict__ pt_ok,
                                                T *__restrict__ W) {
    constexpr int KC = D - 6;
    constexpr int NS = KC * (KC + 1) / 2;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nP) return;
    long long slot = inc_off[p];
    if (slot == inc_off[p + 1]) return;
    const int o0 = pt_start[p], o1 = pt_start[p + 1];
    const bool ok = pt_ok[p] != 0;
    T C[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) C[k] = ok ? pt_Cinv[6 * (size_t)p + k] : T(0);
    for (int o = o0; o < o1; ++o) {
        const int sc = img_shcam[__ldg(J.obrec + o).x];
        if (sc < 0) continue;
        bool first = true;
        for (int o2 = o0; o2 < o && first; ++o2) first = img_shcam[__ldg(J.obrec + o2).x] != sc;
        if (!first) continue;
        T y[3][KC];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int k = 0; k < KC; ++k) y[r][k] = T(0);
        if (ok) {
            for (int o2 = o; o2 < o1; ++o2) {
                const int4 rc = __ldg(J.obrec + o2);
                if (img_shcam[rc.x] != sc) continue;
                ObsOp<T, D, RC, M> op;
                make_op_point_major<T, D, RC>(J, o2, rc, op);
                T jx[6], jc[2 * D];
                op.jx_rows(jx);
                op.jc_rows(jc);
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int k = 0; k < KC; ++k) y[r][k] += jx[r] * jc[6 + k] + jx[3 + r] * jc[D + 6 + k];
            }
        }
        // U = C^-1 Y (C^-1 symmetric, stored 00 01 02 11 12 22)
        T U[3][KC];
#pragma unroll
        for (int k = 0; k < KC; ++k) {
            U[0][k] = C[0] * y[0][k] + C[1] * y[1][k] + C[2] * y[2][k];
            U[1][k] = C[1] * y[0][k] + C[3] * y[1][k] + C[4] * y[2][k];
            U[2][k] = C[2] * y[0][k] + C[4] * y[1][k] + C[5] * y[2][k];
        }
        T *dst = W + (size_t)slot * NS;
        int e = 0;
#pragma unroll
        for (int a = 0; a < KC; ++a)
#pragma unroll
            for (int b = a; b < KC; ++b) {
                dst[e] = y[0][a] * U[0][b] + y[1][a] * U[1][b] + y[2][a] * U[2][b];
                ++e;
            }
        ++slot;
    }
}

// Chunk q (incidences [first, end) of one camera in sorted order) summed in
// order, in FP64. One warp per chunk, one lane per triangle entry.
template <typename T>
__global__ void __launch_bounds__(128) k_sh_chunks(const T *__restrict__ W, const int *__restrict__ inc_sorted,
                                                   const int4 *__restrict__ chunk, int nchunks, int NS,
                                                   double *__restrict__ part) {
    const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= nchunks) return;
    const int4 ch = chunk[q];
    for (int e = lane; e < NS; e += 32) {
        double s = 0.0;
        for (int j = ch.y; j < ch.z; ++j) s += (double)W[(size_t)inc_sorted[j] * NS + e];
        part[(size_t)q * NS + e] = s;
    }
}

// Shared camera c's preconditioner block, rhs and PCG start entries, one
// warp per camera (after the image blocks' own start, k_mf_precond_finish,
// which left the linked images' camera columns out of M, z and the dots).
template <typename T, int D>
__global__ void __launch_bounds__(128) k_sh_precond(const double *__restrict__ img_H,
                                                    const double *__restrict__ img_rhs,
                                                    const int *__restrict__ img_active,
                                                    const int *__restrict__ sh_img_start,
                                                    const int *__restrict__ sh_imgs,
                                                    const int *__restrict__ cam_chunk_off,
                                                    const double *__restrict__ chunk_part,
                                                    const LMState *__restrict__ st, int nsh, int nI,
                                                    T *__restrict__ Minv, T *__restrict__ r, T *__restrict__ z,
                                                    T *__restrict__ p, float *__restrict__ p4,
                                                    double *__restrict__ dots) {
    constexpr int KC = D - 6;
    constexpr int WPB = 4;
    __shared__ double Ls[WPB][KC][KC + 1];
    __shared__ double Ms[WPB][KC][KC + 1];
    __shared__ double rvs[WPB][KC];
    __shared__ double invd_s[WPB][KC];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.x * WPB + wl;
    if (c >= nsh) return;
    double(&L)[KC][KC + 1] = Ls[wl];
    double(&Mi)[KC][KC + 1] = Ms[wl];
    double *rv = rvs[wl];
    double *invd = invd_s[wl];
    const double lam = st->lambda;
    const int i0 = sh_img_start[c], i1 = sh_img_start[c + 1];
    const int owner = sh_imgs[i0];
    const int act = img_active[owner] >> 6;  // the camera's unknown columns (masked parameters off)
    const int q0 = cam_chunk_off[c], q1 = cam_chunk_off[c + 1];
    constexpr int NS = KC * (KC + 1) / 2;
    for (int e = lane; e < KC * KC; e += 32) {
        const int a = e / KC, b = e - a * KC;
        if (b < a) continue;
        double h = 0.0;
        for (int k = i0; k < i1; ++k) {
            const double v = img_H[(size_t)sh_imgs[k] * D * D + (6 + a) * D + 6 + b];
            h += v + (a == b ? lam * v : 0.0);
        }
        const int t = a * KC - a * (a - 1) / 2 + (b - a);  // upper-triangle index
        double w = 0.0;
        for (int q = q0; q < q1; ++q) w += chunk_part[(size_t)q * NS + t];
        double v = h - w;
        const bool on = ((act >> a) & 1) && ((act >> b) & 1);
        if (!on) v = a == b ? 1.0 : 0.0;
        L[a][b] = v;
        L[b][a] = v;
        if (a == b) Mi[a][a] = v;
    }
    if (lane < KC) {
        double s = 0.0;
        if ((act >> lane) & 1)
            for (int k = i0; k < i1; ++k) s += img_rhs[(size_t)sh_imgs[k] * D + 6 + lane];
        rv[lane] = s;
    }
    __syncwarp();
    bool ok = true;
    for (int j = 0; j < KC; ++j) {
        const double d = L[j][j];
        if (!(d > 0.0)) { ok = false; break; }
        const double sd = sqrt(d);
        const double id = 1.0 / sd;
        __syncwarp();
        if (lane == 0) { L[j][j] = sd; invd[j] = id; }
        if (lane > j && lane < KC) L[lane][j] *= id;
        __syncwarp();
        const int m = KC - j - 1;
        for (int idx = lane; idx < m * m; idx += 32) {
            const int a = j + 1 + idx / m, b = j + 1 + idx % m;
            if (b <= a) L[a][b] -= L[a][j] * L[b][j];
        }
        __syncwarp();
    }
    if (ok) {
        double col[KC];
        if (lane < KC) {
            const int cc = lane;
#pragma unroll
            for (int a = 0; a < KC; ++a) {
                double v = a == cc ? 1.0 : 0.0;
#pragma unroll
                for (int k = 0; k < a; ++k) v -= L[a][k] * col[k];
                col[a] = a < cc ? 0.0 : v * invd[a];
            }
#pragma unroll
            for (int a = KC - 1; a >= 0; --a) {
                double v = col[a];
#pragma unroll
                for (int k = a + 1; k < KC; ++k) v -= L[k][a] * col[k];
                col[a] = v * invd[a];
            }
        }
        __syncwarp();
        if (lane < KC)
#pragma unroll
            for (int a = 0; a < KC; ++a) Mi[a][lane] = col[a];
    } else {
        double dl = 0.0;
        if (lane < KC) dl = Mi[lane][lane];
        __syncwarp();
        if (lane < KC)
            for (int a = 0; a < KC; ++a) Mi[a][lane] = (a == lane && dl > 0.0) ? 1.0 / dl : 0.0;
    }
    __syncwarp();
    for (int idx = lane; idx < KC * KC; idx += 32) {
        const int a = idx / KC, b = idx - a * KC;
        const bool on = ((act >> a) & 1) && ((act >> b) & 1);
        if (!on) Mi[a][b] = 0.0;
        Minv[(size_t)owner * D * D + (6 + a) * D + 6 + b] = (T)Mi[a][b];
    }
    __syncwarp();
    double rz = 0.0, rr = 0.0;
    if (lane < KC) {
        double zc = 0.0;
#pragma unroll
        for (int d = 0; d < KC; ++d) zc += Mi[lane][d] * rv[d];
        const T rt = (T)rv[lane], zt = (T)zc;
        for (int k = i0; k < i1; ++k) {
            const int i = sh_imgs[k];
            r[(size_t)i * D + 6 + lane] = rt;
            p[(size_t)i * D + 6 + lane] = zt;
            if (p4) store_dir(p4, nI, i, 6 + lane, (float)zt);
        }
        z[(size_t)owner * D + 6 + lane] = zt;
        rz = (double)rt * (double)zt;
        rr = (double)rt * (double)rt;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        rz += __shfl_xor_sync(0xffffffffu, rz, off);
        rr += __shfl_xor_sync(0xffffffffu, rr, off);
    }
    if (lane == 0) {
        dots[owner] += rz;
        dots[nI + owner] += rr;
    }
}

// q on camera c's columns summed over its images (image order, FP64) and
// written back to every one of them; the owner's p.q partial gains
// p_c . q_c (k_pcg_images_finish left the linked columns out of it).
template <typename T, int D>
__global__ void __launch_bounds__(128) k_sh_qreduce(const int *__restrict__ sh_img_start,
                                                    const int *__restrict__ sh_imgs, int nsh,
                                                    const LMState *__restrict__ st, int nI, const T *__restrict__ p,
                                                    T *__restrict__ q, double *__restrict__ part) {
    constexpr int KC = D - 6;
    if (st->pcg_done) return;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= nsh) return;
    const int i0 = sh_img_start[c], i1 = sh_img_start[c + 1];
    const int owner = sh_imgs[i0];
    double pq = 0.0;
    if (lane < KC) {
        double s = 0.0;
        for (int k = i0; k < i1; ++k) s += (double)q[(size_t)sh_imgs[k] * D + 6 + lane];
        const T qt = (T)s;
        for (int k = i0; k < i1; ++k) q[(size_t)sh_imgs[k] * D + 6 + lane] = qt;
        pq = (double)p[(size_t)owner * D + 6 + lane] * (double)qt;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) pq += __shfl_xor_sync(0xffffffffu, pq, off);
    if (lane == 0) part[2 * nI + owner] += pq;
}

}  // namespace

size_t shared_setup_temp_bytes(int nP, long long ninc) {
    size_t a = 0, bsz = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, a, (long long *)nullptr, (long long *)nullptr, nP + 1);
    const int n = (int)std::max<long long>(1, std::min<long long>(ninc, (1LL << 31) - 1));
    cub::DeviceRadixSort::SortPairs(nullptr, bsz, (int *)nullptr, (int *)nullptr, (int *)nullptr, (int *)nullptr, n);
    return std::max(a, bsz);
}

long long launch_shared_count(const Bufs &b, long long *count, void *temp, size_t temp_bytes, cudaStream_t s) {
    if (b.nP == 0) return 0;
    k_sh_count<<<div_up(b.nP + 1, 128), 128, 0, s>>>(b.pt_start, b.ob_img, b.sh.img_shcam, b.nP, count);
    SFMBA_LAUNCH_CHECK();
    size_t tb = temp_bytes;
    SFMBA_CUDA(cub::DeviceScan::ExclusiveSum(temp, tb, count, b.sh.inc_off, b.nP + 1, s));
    long long ninc = 0;
    SFMBA_CUDA(cudaMemcpyAsync(&ninc, b.sh.inc_off + b.nP, sizeof(long long), cudaMemcpyDeviceToHost, s));
    SFMBA_CUDA(cudaStreamSynchronize(s));
    return ninc;
}

void launch_shared_sort(const Bufs &b, int *key, int *val, int *key2, int *cam_counts, void *temp,
                        size_t temp_bytes, cudaStream_t s) {
    const SharedBufs &sh = b.sh;
    SFMBA_CUDA(cudaMemsetAsync(cam_counts, 0, sizeof(int) * (size_t)sh.nsh, s));
    if (sh.ninc <= 0) return;
    k_sh_emit<<<div_up(b.nP, 128), 128, 0, s>>>(b.pt_start, b.ob_img, sh.img_shcam, sh.inc_off, b.nP, key, val);
    SFMBA_LAUNCH_CHECK();
    int bits = 1;
    while ((1 << bits) < sh.nsh) ++bits;
    size_t tb = temp_bytes;
    SFMBA_CUDA(cub::DeviceRadixSort::SortPairs(temp, tb, key, key2, val, sh.inc_sorted, (int)sh.ninc, 0, bits, s));
    k_sh_key_counts<<<div_up(sh.ninc, 256), 256, 0, s>>>(key2, sh.ninc, cam_counts);
    SFMBA_LAUNCH_CHECK();
}

void launch_shared_precond(const Bufs &b, cudaStream_t s) {
    const SharedBufs &sh = b.sh;
    if (sh.nsh == 0) return;
    dispatch_TDR(b, [&](auto t, auto dc, auto rc, auto mc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        if constexpr (D > 6) {
            constexpr int KC = D - 6;
            constexpr int NS = KC * (KC + 1) / 2;
            if (sh.ninc > 0) {
                k_sh_inc<T, D, decltype(rc)::value, -1><<<div_up(b.nP, 128), 128, 0, s>>>(
                    jac_src<T>(b), b.pt_start, sh.img_shcam, sh.inc_off, b.nP, (const T *)b.pt_Cinv, b.pt_ok,
                    (T *)sh.inc_W);
                SFMBA_LAUNCH_CHECK();
                k_sh_chunks<T><<<div_up(sh.nchunks, 4), 128, 0, s>>>((const T *)sh.inc_W, sh.inc_sorted, sh.chunk,
                                                                     sh.nchunks, NS, sh.chunk_part);
                SFMBA_LAUNCH_CHECK();
            }
            k_sh_precond<T, D><<<div_up(sh.nsh, 4), 128, 0, s>>>(
                b.img_H, b.img_rhs, b.img_active, sh.sh_img_start, sh.sh_imgs, sh.cam_chunk_off, sh.chunk_part,
                b.state, sh.nsh, b.nI, (T *)b.pcg_Minv, (T *)b.pcg_r, (T *)b.pcg_z, (T *)b.pcg_p,
                std::is_same<T, float>::value ? b.pcg_p4 : nullptr, b.pcg_part);
            SFMBA_LAUNCH_CHECK();
        } else {
            throw Error(SFMBA_ERR_INTERNAL, "shared cameras without camera columns");
        }
    });
}

void launch_shared_qreduce(const Bufs &b, cudaStream_t s) {
    const SharedBufs &sh = b.sh;
    if (sh.nsh == 0) return;
    dispatch_D(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        if constexpr (D > 6) {
            auto run = [&](auto t) {
                using T = decltype(t);
                k_sh_qreduce<T, D><<<div_up(sh.nsh, 4), 128, 0, s>>>(sh.sh_img_start, sh.sh_imgs, sh.nsh, b.state,
                                                                     b.nI, (const T *)b.pcg_p, (T *)b.pcg_q,
                                                                     b.pcg_part);
                SFMBA_LAUNCH_CHECK();
            };
            if (b.mixed) run(0.0f);
            else run(0.0);
        }
    });
}

}  // namespace sfmba
