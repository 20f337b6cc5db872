// Local bundle-adjustment windows (sfm-reconstruction's BaScope::Local)
// built from a reconstruction in progress, many centres per call.
//
// Follows crates/sfm-reconstruction/src/lib.rs:1336-1473 for one centre:
//   * free points: every point with a track of at least two elements one of
//     which is in the centre image (:1345-1352);
//   * co-visibility: per registered image other than the centre, the number
//     of track elements of those points in it; ranked by count (descending)
//     then image index, the first num_free_neighbours join the centre as
//     free images (:1353-1376, LOCAL_BA_NUM_IMAGES = 6 at :1320);
//   * window images: every registered image with a track element of a free
//     point, in index order; fewer than two means no window (:1385-1406);
//   * cameras in order of first use by the window images (:1408-1420);
//   * fixed poses: the seed image, every image outside the free set and
//     every pose the caller pinned; if none is fixed, the first window image
//     (:1427-1456);
//   * observations: the free points in order, each point's track elements in
//     track order whose image is in the window (:1458-1473); none means no
//     window;
//   * intrinsics held (local bundles run with IntrinsicsMode::Fixed, :708-719)
//     with the principal point masked (default_fixed_params_mask, :1489).
// The windows are independent, so they are built on parallel host threads.
#include <algorithm>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sfmba.h"

namespace sfmba {

void record_error(const char *message);

namespace {

struct BadInput {
    std::string what;
};

int dof_of(int m) {
    switch (m) {
    case SFMBA_SIMPLE_PINHOLE: return 3;
    case SFMBA_PINHOLE: return 4;
    case SFMBA_SIMPLE_RADIAL: return 4;
    case SFMBA_RADIAL: return 5;
    case SFMBA_OPENCV: return 8;
    case SFMBA_OPENCV_FISHEYE: return 8;
    default: return 0;
    }
}

struct Window {
    std::vector<int32_t> image_ids, camera_ids, point_ids, camera_of_image, obs_image, obs_point;
    std::vector<double> obs_xy;
    std::vector<uint8_t> fixed_poses;
    bool empty() const { return obs_image.empty(); }
};

Window build_window(const sfmba_reconstruction &R, int seed, int num_free, int center) {
    Window W;
    const int64_t nI = R.num_images, nP = R.num_points;
    const int64_t *off = R.track_offsets;
    std::vector<int32_t> pts;
    for (int64_t p = 0; p < nP; ++p) {
        if (off[p + 1] - off[p] < 2) continue;
        bool hit = false;
        for (int64_t e = off[p]; e < off[p + 1] && !hit; ++e) hit = R.track_image[e] == center;
        if (hit) pts.push_back((int32_t)p);
    }
    std::vector<int64_t> covis(nI, 0);
    std::vector<uint8_t> seen(nI, 0);
    for (int32_t p : pts)
        for (int64_t e = off[p]; e < off[p + 1]; ++e) {
            const int img = R.track_image[e];
            if (!R.registered[img]) continue;
            seen[img] = 1;
            if (img != center) covis[img] += 1;
        }
    std::vector<std::pair<int64_t, int>> ranked;
    for (int64_t i = 0; i < nI; ++i)
        if (covis[i] > 0) ranked.push_back({covis[i], (int)i});
    std::sort(ranked.begin(), ranked.end(), [](const std::pair<int64_t, int> &a, const std::pair<int64_t, int> &b) {
        return a.first != b.first ? a.first > b.first : a.second < b.second;
    });
    std::vector<uint8_t> free_img(nI, 0);
    for (size_t k = 0; k < ranked.size() && (int64_t)k < num_free; ++k) free_img[ranked[k].second] = 1;
    free_img[center] = 1;
    std::vector<int32_t> pos(nI, -1);
    for (int64_t i = 0; i < nI; ++i)
        if (seen[i]) {
            pos[i] = (int32_t)W.image_ids.size();
            W.image_ids.push_back((int32_t)i);
        }
    if (W.image_ids.size() < 2) return Window();
    std::vector<int32_t> cam_pos(R.num_cameras, -1);
    for (int32_t i : W.image_ids) {
        const int c = R.camera_of_image[i];
        if (cam_pos[c] < 0) {
            cam_pos[c] = (int32_t)W.camera_ids.size();
            W.camera_ids.push_back(c);
        }
        W.camera_of_image.push_back(cam_pos[c]);
    }
    bool any_fixed = false;
    for (int32_t i : W.image_ids) {
        const bool f = i == seed || !free_img[i] || (R.pose_fixed && R.pose_fixed[i]);
        W.fixed_poses.push_back(f ? 1 : 0);
        any_fixed = any_fixed || f;
    }
    if (!any_fixed) W.fixed_poses[0] = 1;
    for (size_t cp = 0; cp < pts.size(); ++cp) {
        const int32_t p = pts[cp];
        for (int64_t e = off[p]; e < off[p + 1]; ++e) {
            const int32_t ci = pos[R.track_image[e]];
            if (ci < 0) continue;
            W.obs_image.push_back(ci);
            W.obs_point.push_back((int32_t)cp);
            W.obs_xy.push_back(R.track_xy[2 * e]);
            W.obs_xy.push_back(R.track_xy[2 * e + 1]);
        }
    }
    if (W.obs_image.empty()) return Window();
    W.point_ids = std::move(pts);
    return W;
}

void validate(const sfmba_reconstruction *R, int seed, int num_free, int num_centers, const int32_t *centers) {
    if (!R) throw BadInput{"reconstruction is NULL"};
    if (R->num_images < 0 || R->num_cameras < 0 || R->num_points < 0) throw BadInput{"negative size"};
    if (R->num_images > (1 << 30) || R->num_points > (1LL << 31) - 1) throw BadInput{"reconstruction too large"};
    if (num_free < 0) throw BadInput{"num_free_neighbours < 0"};
    if (num_centers < 0 || (num_centers > 0 && !centers)) throw BadInput{"bad centres"};
    if (seed < -1 || seed >= R->num_images) throw BadInput{"seed_image out of range"};
    auto need = [](const void *p, int64_t n, const char *name) {
        if (n > 0 && !p) throw BadInput{std::string(name) + " is NULL"};
    };
    need(R->camera_of_image, R->num_images, "camera_of_image");
    need(R->registered, R->num_images, "registered");
    need(R->poses, R->num_images, "poses");
    need(R->camera_model, R->num_cameras, "camera_model");
    need(R->camera_params, R->num_cameras, "camera_params");
    need(R->points, R->num_points, "points");
    if (!R->track_offsets) throw BadInput{"track_offsets is NULL"};
    if (R->track_offsets[0] != 0) throw BadInput{"track_offsets[0] != 0"};
    for (int64_t p = 0; p < R->num_points; ++p)
        if (R->track_offsets[p + 1] < R->track_offsets[p]) throw BadInput{"track_offsets decrease"};
    const int64_t ne = R->track_offsets[R->num_points];
    need(R->track_image, ne, "track_image");
    need(R->track_xy, ne, "track_xy");
    for (int64_t e = 0; e < ne; ++e)
        if (R->track_image[e] < 0 || R->track_image[e] >= R->num_images)
            throw BadInput{"track_image[" + std::to_string(e) + "] out of range"};
    for (int64_t i = 0; i < R->num_images; ++i)
        if (R->camera_of_image[i] < 0 || R->camera_of_image[i] >= R->num_cameras)
            throw BadInput{"camera_of_image[" + std::to_string(i) + "] out of range"};
    for (int64_t c = 0; c < R->num_cameras; ++c)
        if (dof_of(R->camera_model[c]) == 0) throw BadInput{"camera " + std::to_string(c) + " has an unknown model id"};
    for (int k = 0; k < num_centers; ++k)
        if (centers[k] < 0 || centers[k] >= R->num_images)
            throw BadInput{"centers[" + std::to_string(k) + "] out of range"};
}

template <typename F>
void for_each_parallel(int n, F &&f) {
    const int nt = std::max(1, std::min<int>(n, (int)std::thread::hardware_concurrency()));
    if (nt <= 1) {
        for (int k = 0; k < n; ++k) f(k);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            for (int k = t; k < n; k += nt) f(k);
        });
    for (auto &x : th) x.join();
}

}  // namespace

}  // namespace sfmba

using namespace sfmba;

extern "C" int sfmba_local_windows(const sfmba_reconstruction *rec, int32_t seed_image, int32_t num_free_neighbours,
                                   int32_t num_centers, const int32_t *centers, int64_t *counts_out,
                                   sfmba_window_buffers *windows) {
    try {
        validate(rec, seed_image, num_free_neighbours, num_centers, centers);
        if (num_centers > 0 && !counts_out) throw BadInput{"counts_out is NULL"};
        std::vector<Window> ws(num_centers);
        for_each_parallel(num_centers, [&](int k) {
            ws[k] = build_window(*rec, seed_image, num_free_neighbours, centers[k]);
        });
        for (int k = 0; k < num_centers; ++k) {
            const Window &W = ws[k];
            const int64_t got[4] = {W.empty() ? 0 : (int64_t)W.image_ids.size(),
                                    W.empty() ? 0 : (int64_t)W.camera_ids.size(),
                                    W.empty() ? 0 : (int64_t)W.point_ids.size(), (int64_t)W.obs_image.size()};
            if (windows) {  // the buffers were sized by a previous sizing call: check the sizes still hold
                for (int j = 0; j < 4; ++j)
                    if (counts_out[4 * k + j] != got[j])
                        throw BadInput{"window " + std::to_string(k) + ": counts_out differs from the sizing call"};
            }
            std::memcpy(counts_out + 4 * k, got, sizeof(got));
        }
        if (!windows) {
            record_error("");
            return SFMBA_OK;
        }
        for_each_parallel(num_centers, [&](int k) {
            const Window &W = ws[k];
            if (W.empty()) return;
            sfmba_window_buffers &B = windows[k];
            const size_t nI = W.image_ids.size(), nC = W.camera_ids.size(), nP = W.point_ids.size();
            const size_t nO = W.obs_image.size();
            auto cp = [](auto *dst, const auto &src) {
                if (dst && !src.empty()) std::memcpy(dst, src.data(), sizeof(src[0]) * src.size());
            };
            cp(B.image_ids, W.image_ids);
            cp(B.camera_ids, W.camera_ids);
            cp(B.point_ids, W.point_ids);
            cp(B.camera_of_image, W.camera_of_image);
            cp(B.obs_image, W.obs_image);
            cp(B.obs_point, W.obs_point);
            cp(B.obs_xy, W.obs_xy);
            cp(B.fixed_poses, W.fixed_poses);
            for (size_t c = 0; c < nC; ++c) {
                const int src = W.camera_ids[c], m = rec->camera_model[src];
                if (B.camera_model) B.camera_model[c] = m;
                if (B.camera_params) std::memcpy(B.camera_params + 8 * c, rec->camera_params + 8 * (size_t)src, 64);
                if (B.fixed_cameras) B.fixed_cameras[c] = 1;
                if (B.fixed_camera_params) {
                    // intrinsics.rs:33-61: principal point (1,2) for the f-only models, (2,3) otherwise
                    std::memset(B.fixed_camera_params + 8 * c, 0, 8);
                    const int a = (m == SFMBA_SIMPLE_PINHOLE || m == SFMBA_SIMPLE_RADIAL || m == SFMBA_RADIAL) ? 1 : 2;
                    B.fixed_camera_params[8 * c + a] = 1;
                    B.fixed_camera_params[8 * c + a + 1] = 1;
                }
            }
            for (size_t i = 0; i < nI; ++i)
                if (B.poses) std::memcpy(B.poses + 7 * i, rec->poses + 7 * (size_t)W.image_ids[i], 56);
            for (size_t p = 0; p < nP; ++p)
                if (B.points) std::memcpy(B.points + 3 * p, rec->points + 3 * (size_t)W.point_ids[p], 24);
            (void)nO;
        });
        record_error("");
        return SFMBA_OK;
    } catch (const BadInput &e) {
        record_error(("sfmba_local_windows: " + e.what).c_str());
        return SFMBA_ERR_INVALID_ARGUMENT;
    } catch (const std::exception &e) {
        record_error(e.what());
        return SFMBA_ERR_INTERNAL;
    }
}
