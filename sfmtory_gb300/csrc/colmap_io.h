// COLMAP plain-text sparse model (cameras.txt / images.txt / points3D.txt),
// read and written as crates/sfm-io/src/colmap.rs does: the same tokens,
// the same number formats on output, the same rejection of malformed
// lines. Host code; the refine driver that uses it is in solver.cu.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <utility>
#include <vector>

namespace sfmba {

struct ColmapCamera {
    uint32_t id = 0;
    int model = 0;            // sfmba_camera_model
    uint32_t width = 0, height = 0;
    double params[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

struct ColmapImage {
    uint32_t id = 0;
    double q[4] = {1, 0, 0, 0};  // qw qx qy qz
    double t[3] = {0, 0, 0};
    uint32_t camera_id = 0;
    std::string name;
    std::vector<std::pair<float, float>> keypoints;
    std::vector<int64_t> point3d_ids;  // -1: none
};

struct ColmapPoint {
    uint64_t id = 0;
    double xyz[3] = {0, 0, 0};
    uint8_t color[3] = {0, 0, 0};
    double error = 0.0;
    std::vector<std::pair<uint32_t, uint32_t>> track;  // (image id, keypoint index)
};

// crates/sfm-core/src/model.rs (`Reconstruction`), maps in id order.
struct ColmapModel {
    std::map<uint32_t, ColmapCamera> cameras;
    std::map<uint32_t, ColmapImage> images;
    std::map<uint64_t, ColmapPoint> points;

    // Reconstruction::mean_reprojection_error (model.rs:84-97): the points'
    // stored errors weighted by track length.
    double mean_reprojection_error() const;
};

// Throws sfmba::Error (SFMBA_ERR_INVALID_ARGUMENT) on a missing file or a
// malformed line, with the file and the reason in the message.
ColmapModel colmap_read(const std::string &dir);
void colmap_write(const ColmapModel &m, const std::string &dir);

}  // namespace sfmba
