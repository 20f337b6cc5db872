// Launchers of the observation passes run once per linearisation (point
// and image blocks, preconditioner, back-substitution) and the record
// packing; the per-PCG-iteration passes are in k_mf_pcg.cu.
#include "mf_passes.cuh"

namespace sfmba {

namespace {

// The padded FP32 mirror of p (NULL for FP64).
template <typename T>
void *pcg_p4_of(const Bufs &b) {
    return std::is_same<T, float>::value ? (void *)b.pcg_p4 : nullptr;
}

// Packed {image, point, x, y} records of both observation orders.
__global__ void k_pack_records(const int *img_obs, const int *ob_img, const int *ob_pt, const double2 *ob_xy,
                               long long nO, int4 *obrec, int4 *isrec) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= nO) return;
    if (obrec) {  // point-major records: PCG solver only
        const double2 a = ob_xy[k];
        obrec[k] = make_int4(ob_img[k], ob_pt[k], __float_as_int((float)a.x), __float_as_int((float)a.y));
    }
    const int o = img_obs[k];
    const double2 b = ob_xy[o];
    isrec[k] = make_int4(ob_img[o], ob_pt[o], __float_as_int((float)b.x), __float_as_int((float)b.y));
}

}  // namespace

void launch_mf_prepare(const Bufs &b, cudaStream_t s) {
    if (b.nO > 0) {
        k_pack_records<<<div_up(b.nO, 256), 256, 0, s>>>(b.img_obs, b.ob_img, b.ob_pt, b.ob_xy, b.nO, b.obrec, b.isrec);
        SFMBA_LAUNCH_CHECK();
    }
}

void launch_mf_point_reduce(const Bufs &b, cudaStream_t s) {
    if (b.npchunks == 0) return;
    dispatch_TDR(b, [&](auto t, auto dc, auto rc, auto mc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        k_mf_point_reduce<T, D, decltype(rc)::value, decltype(mc)::value><<<warps_grid(b.npchunks, 256), 256, 0, s>>>(
            jac_src<T>(b), b.ob_valid, b.img_free, b.pchunk, b.npchunks, (T *)b.pt_C, (T *)b.pt_g, b.pt_nfree);
    });
    SFMBA_LAUNCH_CHECK();
}

void launch_mf_image_blocks(const Bufs &b, cudaStream_t s) {
    dispatch_TDR(b, [&](auto t, auto dc, auto rc, auto mc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        if (b.n_iachunks > 0) {
            const int th = 32 * accum_warps<T>();
            k_mf_image_accum<T, D, decltype(rc)::value, 0, decltype(mc)::value><<<warps_grid(b.n_iachunks, th), th, 0, s>>>(
                jac_src<T>(b), b.iachunk, b.n_iachunks, (const T *)b.pt_Cinv, (const T *)b.pt_h, b.pt_ok,
                (T *)b.ipart2);
            SFMBA_LAUNCH_CHECK();
        }
        k_mf_image_finish0<T, D><<<div_up(b.nI, 4), 128, 0, s>>>((const T *)b.ipart2, b.iachunk_off, b.nI,
                                                                b.img_live, b.img_H, b.img_b,
                                                                D * (D + 1) / 2 + D);
        SFMBA_LAUNCH_CHECK();
    });
}

// H_i, b_i from the stored records (dense and batched paths): the same
// register-tiled accumulation over image-aligned chunks, Jacobians read
// from the records (RC = false) in the records' precision.
void launch_image_blocks_records(const Bufs &b, cudaStream_t s) {
    dispatch_D(b.D, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        auto run = [&](auto t) {
            using T = decltype(t);
            if (b.n_iachunks > 0) {
                const int th = 32 * accum_warps<T>();
                k_mf_image_accum<T, D, false, 0><<<warps_grid(b.n_iachunks, th), th, 0, s>>>(
                    jac_src<T>(b), b.iachunk, b.n_iachunks, (const T *)b.pt_Cinv, (const T *)b.pt_h, b.pt_ok,
                    (T *)b.ipart2);
                SFMBA_LAUNCH_CHECK();
            }
            k_mf_image_finish0<T, D><<<div_up(b.nI, 4), 128, 0, s>>>((const T *)b.ipart2, b.iachunk_off, b.nI,
                                                                    b.img_live, b.img_H, b.img_b,
                                                                    D * (D + 1) / 2 + D);
            SFMBA_LAUNCH_CHECK();
        };
        if (b.mixed) run(0.0f);
        else run(0.0);
    });
}

void launch_mf_precond(const Bufs &b, cudaStream_t s) {
    dispatch_TDR(b, [&](auto t, auto dc, auto rc, auto mc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        if (b.n_iachunks > 0) {
            const int th = 32 * accum_warps<T>();
            k_mf_image_accum<T, D, decltype(rc)::value, 1, decltype(mc)::value><<<warps_grid(b.n_iachunks, th), th, 0, s>>>(
                jac_src<T>(b), b.iachunk, b.n_iachunks, (const T *)b.pt_Cinv, (const T *)b.pt_h, b.pt_ok,
                (T *)b.ipart2);
            SFMBA_LAUNCH_CHECK();
        }
        k_mf_precond_finish<T, D><<<div_up(b.nI, 4), 128, 0, s>>>((const T *)b.ipart2, b.iachunk_off, b.img_H, b.img_b,
                                                       b.img_active, b.img_pmask, b.state, b.nI, b.img_rhs, (T *)b.pcg_Minv,
                                                       (T *)b.pcg_x, (T *)b.pcg_r, (T *)b.pcg_z, (T *)b.pcg_p,
                                                       (T *)pcg_p4_of<T>(b), b.pcg_part, D * (D + 1) / 2 + D,
                                                       std::is_same<T, float>::value ? b.img_Hf : nullptr);
        SFMBA_LAUNCH_CHECK();
    });
}

void launch_mf_precond_fused(const Bufs &b, cudaStream_t s) {
    dispatch_TDR(b, [&](auto t, auto dc, auto rc, auto mc) {
        using T = decltype(t);
        constexpr int D = decltype(dc)::value;
        constexpr int NV = D * (D + 1) / 2 + D;
        if constexpr (std::is_same<T, float>::value) {
            if (b.n_iachunks > 0) {
                const int th = 32 * accum_warps<T>();
                k_mf_image_accum<T, D, decltype(rc)::value, 2, decltype(mc)::value>
                    <<<warps_grid(b.n_iachunks, th), th, 0, s>>>(jac_src<T>(b), b.iachunk, b.n_iachunks,
                                                                 (const T *)b.pt_Cinv, (const T *)b.pt_h, b.pt_ok,
                                                                 (T *)b.ipart2);
                SFMBA_LAUNCH_CHECK();
            }
            k_mf_image_finish0<T, D><<<div_up(b.nI, 4), 128, 0, s>>>((const T *)b.ipart2, b.iachunk_off, b.nI,
                                                                    b.img_live, b.img_H, b.img_b, 2 * NV);
            SFMBA_LAUNCH_CHECK();
            k_mf_precond_finish<T, D><<<div_up(b.nI, 4), 128, 0, s>>>(
                (const T *)b.ipart2 + NV, b.iachunk_off, b.img_H, b.img_b, b.img_active, b.img_pmask, b.state, b.nI, b.img_rhs,
                (T *)b.pcg_Minv, (T *)b.pcg_x, (T *)b.pcg_r, (T *)b.pcg_z, (T *)b.pcg_p, (T *)pcg_p4_of<T>(b),
                b.pcg_part, 2 * NV, b.img_Hf);
            SFMBA_LAUNCH_CHECK();
        } else {
            throw Error(SFMBA_ERR_INTERNAL, "the fused image pass is FP32 only");
        }
    });
}

void launch_mf_backsub(const Bufs &b, const double *delta_slot, cudaStream_t s) {
    launch_gather_delta(b, delta_slot, s);
    if (b.nP > 0)
        SFMBA_CUDA(cudaMemcpyAsync(b.points_trial, b.points, sizeof(double) * 3 * (size_t)b.nP,
                                   cudaMemcpyDeviceToDevice, s));
    if (b.npchunks > 0) {
        dispatch_TDR(b, [&](auto t, auto dc, auto rc, auto mc) {
            using T = decltype(t);
            constexpr int D = decltype(dc)::value;
            k_mf_backsub<T, D, decltype(rc)::value, decltype(mc)::value><<<warps_grid(b.npchunks, 256), 256, 0, s>>>(
                jac_src<T>(b), b.pchunk, b.npchunks, (const T *)b.img_delta, (const T *)b.pt_Cinv,
                (const T *)b.pt_g, b.pt_ok, b.points, b.points_trial);
        });
        SFMBA_LAUNCH_CHECK();
    }
    launch_update_images(b, delta_slot, s);
}

}  // namespace sfmba
