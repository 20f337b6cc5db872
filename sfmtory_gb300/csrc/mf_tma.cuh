// PCG point pass with its record stream staged by the Tensor Memory
// Accelerator.
//
// The same sums as k_mf_points (u_p = C_p^-1 sum_o Jx~^T (Jc~_o p_img(o)),
// MvOp operator, segmented warp scan with a carry). The packed records of
// each 32-observation round (16 bytes per observation, contiguous in
// point-major order) arrive by one bulk copy (cp.async.bulk) into a ring of
// shared-memory buffers, kTmaAhead rounds ahead, completed through
// transaction-counting mbarriers, so their DRAM latency leaves the dependent
// chain record -> gathers -> arithmetic without holding registers; the
// per-image constants, the direction vector and the point are gathered by
// the lanes' own loads through L1 (neighbouring lanes share images, so most
// of them hit). It is one of the autotuner's candidates. Measured on the
// 2000-camera problem's point pass: this form 92 us, the register-prefetch
// form (point_chunk with PF) 81 us; with the gathers as per-lane L1-caching
// asynchronous copies into shared memory one round ahead 150 us; with the
// image rows gathered by TMA (tile::gather4, which bypasses L1, so every
// observation fetches its 128-byte row from L2) 307 us. Every mbarrier wait
// is bounded: a wait that gives up counts in LMState::wait_timeouts (the
// host fails the solve with an internal error), ends the PCG solve and lets
// the warp's copies in flight land before it exits.
#pragma once

#include <cuda.h>

#include "mf_passes.cuh"

namespace sfmba {

namespace {

constexpr int kTmaAhead = 4;                  // record rounds in flight ahead of the one computed
constexpr int kTmaRing = kTmaAhead + 1;       // record buffers per warp
constexpr long long kTmaMaxPolls = 1LL << 22;  // bound of every mbarrier wait

constexpr int kTmaWarps = 8;                   // warps per block (four blocks per SM)

struct TmaRecRing {
    alignas(128) int4 rec[kTmaRing][32];  // packed records {image, point, x, y}
    alignas(8) unsigned long long bar[kTmaRing];
};

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Earlier generic-proxy accesses to shared memory before later async-proxy writes.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void bulk_to_shared(unsigned dst, const void *src, unsigned bytes, unsigned bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
// Every lane polls (each gets the barrier's acquire); true when all saw the
// phase complete within the bound.
__device__ __forceinline__ bool warp_wait(unsigned bar, unsigned parity) {
    bool ok = false;
    for (long long k = 0; k < kTmaMaxPolls; ++k)
        if (mbar_try_wait(bar, parity)) {
            ok = true;
            break;
        }
    return __all_sync(0xffffffffu, ok);
}

template <int D, int M>
__global__ void __launch_bounds__(32 * kTmaWarps, 4)
    k_mf_points_tma(JacSrc<float> J, const int *__restrict__ pchunk, int nchunks, const float *__restrict__ pt_Cinv,
                    const unsigned char *__restrict__ pt_ok, const float *__restrict__ p4, LMState *__restrict__ st,
                    float *__restrict__ u) {
    constexpr int NW = kTmaWarps;
    __shared__ TmaRecRing ring[NW];
    if (st->pcg_done) return;
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int warp = blockIdx.x * NW + wl;
    if (warp >= nchunks) return;
    TmaRecRing &W = ring[wl];
    const int cs = pchunk[warp], ce = pchunk[warp + 1];
    const int R = (ce - cs + 31) >> 5;
    if (R <= 0) return;
    unsigned bar[kTmaRing];
#pragma unroll
    for (int k = 0; k < kTmaRing; ++k) bar[k] = smem_addr(&W.bar[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < kTmaRing; ++k) mbar_init(bar[k]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    auto count = [&](int r) { return min(32, ce - cs - 32 * r); };
    auto issue = [&](int r) {  // lane 0: round r's records into ring buffer r % kTmaRing
        const int b = r % kTmaRing, n = count(r);
        fence_proxy_async();
        mbar_expect_tx(bar[b], 16u * n);
        bulk_to_shared(smem_addr(W.rec[b]), J.obrec + cs + 32 * r, 16u * n, bar[b]);
    };
    // Rounds [waited, issued) have records in flight (waited for in round
    // order); a wait that gives up drains them before the warp exits.
    int issued = 0, waited = 0;
    auto fail = [&] {
        if (lane == 0) {
            atomicAdd(&st->wait_timeouts, 1);
            st->pcg_done = 1;
        }
        for (int r = waited; r < issued; ++r) (void)warp_wait(bar[r % kTmaRing], (r / kTmaRing) & 1);
    };
    auto wait_rec = [&](int r) {
        const bool ok = warp_wait(bar[r % kTmaRing], (r / kTmaRing) & 1);
        if (ok) waited = r + 1;
        return ok;
    };
    if (lane == 0)
        for (int r = 0; r < kTmaAhead && r < R; ++r) issue(r);
    issued = min(kTmaAhead, R);
    if (!wait_rec(0)) return fail();

    float carry[3] = {0.f, 0.f, 0.f};
    int carry_pt = -1;
    for (int r = 0; r < R; ++r) {
        if (r + kTmaAhead < R) {  // its buffer was last used by round r - 1, done
            if (lane == 0) issue(r + kTmaAhead);
            issued = r + kTmaAhead + 1;
        }
        if (r + 1 < R && !wait_rec(r + 1)) return fail();  // lane 31 reads its first record
        const int n = count(r);
        const bool valid = lane < n;
        int4 rc = make_int4(0, -1, 0, 0);
        float v[3] = {0.f, 0.f, 0.f};
        if (valid) {
            rc = W.rec[r % kTmaRing][lane];
            float pv[D];
            load_image_vec<float, D>(nullptr, p4, rc.x, J.nI, pv);
            MvOp<D, M> op;
            op.build(J, rc.x, rc.y, rc);
            float s0, s1;
            op.jc_dot(pv, s0, s1);
            op.jx_t(s0, s1, v);
        }
        // Segmented scan of the round, as point_chunk does.
        const int pt = rc.y;
        if (valid && lane == 0 && pt == carry_pt) {
#pragma unroll
            for (int k = 0; k < 3; ++k) v[k] += carry[k];
        }
        const int prev = __shfl_up_sync(0xffffffffu, pt, 1);
        seg_scan<float, 3>(v, lane == 0 || pt != prev, lane);
        int next = __shfl_down_sync(0xffffffffu, pt, 1);
        if (lane == 31) next = (r + 1 < R) ? W.rec[(r + 1) % kTmaRing][0].y : -1;
        const bool tail = valid && next != pt;
        if (tail) {
            float u0 = 0.f, u1 = 0.f, u2 = 0.f;
            if (pt_ok[pt]) {
                const float *Ci = pt_Cinv + 6 * (size_t)pt;
                u0 = Ci[0] * v[0] + Ci[1] * v[1] + Ci[2] * v[2];
                u1 = Ci[1] * v[0] + Ci[3] * v[1] + Ci[4] * v[2];
                u2 = Ci[2] * v[0] + Ci[4] * v[1] + Ci[5] * v[2];
            }
            reinterpret_cast<float4 *>(u)[pt] = make_float4(u0, u1, u2, 0.0f);
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) carry[k] = __shfl_sync(0xffffffffu, v[k], 31);
        carry_pt = __shfl_sync(0xffffffffu, (valid && !tail) ? pt : -1, 31);
        __syncwarp();  // every lane is done with round r's buffers before they are refilled
    }
}

}  // namespace

}  // namespace sfmba
