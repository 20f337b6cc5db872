// COLMAP text model reader/writer (crates/sfm-io/src/colmap.rs:24-305).
#include "colmap_io.h"

#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <limits>
#include <sstream>
#include <type_traits>

#include "common.cuh"

namespace sfmba {

namespace {

const char *const kModelNames[6] = {"SIMPLE_PINHOLE", "PINHOLE", "SIMPLE_RADIAL", "RADIAL", "OPENCV",
                                    "OPENCV_FISHEYE"};

[[noreturn]] void parse_fail(const char *context, const std::string &message) {
    throw Error(SFMBA_ERR_INVALID_ARGUMENT, std::string("parse error in ") + context + ": " + message);
}

std::string read_file(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "cannot read " + path);
    std::ostringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

void write_file(const std::string &path, const std::string &text) {
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "cannot write " + path);
    f << text;
    if (!f) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "cannot write " + path);
}

// str::lines() then trim(): lines split at '\n' (a trailing '\r' removed),
// surrounding whitespace dropped.
std::vector<std::string> trimmed_lines(const std::string &text) {
    std::vector<std::string> out;
    size_t s = 0;
    while (s < text.size()) {
        size_t e = text.find('\n', s);
        if (e == std::string::npos) e = text.size();
        size_t a = s, b = e;
        if (b > a && text[b - 1] == '\r') --b;
        while (a < b && std::isspace((unsigned char)text[a])) ++a;
        while (b > a && std::isspace((unsigned char)text[b - 1])) --b;
        out.emplace_back(text, a, b - a);
        s = e + 1;
    }
    return out;
}

std::vector<std::string> split_ws(const std::string &line) {
    std::vector<std::string> t;
    std::istringstream ss(line);
    std::string w;
    while (ss >> w) t.push_back(w);
    return t;
}

// Integer parsing as Rust's str::parse: optional sign ('-' only for signed
// types), decimal digits, in range; nothing else.
template <typename T>
bool parse_int(const std::string &s, T &out) {
    size_t i = 0;
    bool neg = false;
    if (i < s.size() && (s[i] == '+' || s[i] == '-')) {
        neg = s[i] == '-';
        ++i;
    }
    if (i == s.size()) return false;
    if (neg && !std::is_signed<T>::value) return false;
    unsigned long long v = 0;
    for (; i < s.size(); ++i) {
        if (s[i] < '0' || s[i] > '9') return false;
        const unsigned d = (unsigned)(s[i] - '0');
        if (v > (~0ull - d) / 10) return false;
        v = v * 10 + d;
    }
    if (std::is_signed<T>::value) {
        const unsigned long long lim = (unsigned long long)std::numeric_limits<T>::max() + (neg ? 1 : 0);
        if (v > lim) return false;
        out = neg ? (T)(-(long long)(v - 1) - 1) : (T)v;
    } else {
        if (v > (unsigned long long)std::numeric_limits<T>::max()) return false;
        out = (T)v;
    }
    return true;
}

// Float parsing as Rust's str::parse: decimal (with exponent), inf,
// infinity, nan (any case), optional sign; no hexadecimal form.
template <typename T>
bool parse_float(const std::string &s, T &out) {
    if (s.empty()) return false;
    size_t i = (s[0] == '+' || s[0] == '-') ? 1 : 0;
    if (i + 1 < s.size() && s[i] == '0' && (s[i + 1] == 'x' || s[i + 1] == 'X')) return false;
    std::string low;
    for (size_t k = i; k < s.size(); ++k) low += (char)std::tolower((unsigned char)s[k]);
    if (low.compare(0, 3, "nan") == 0 && low != "nan") return false;  // no nan(...) payloads
    errno = 0;
    char *end = nullptr;
    const double v = std::is_same<T, float>::value ? (double)std::strtof(s.c_str(), &end)
                                                   : std::strtod(s.c_str(), &end);
    if (end != s.c_str() + s.size()) return false;
    out = (T)v;
    return true;
}

// Rust's `{:.N}` of an f64: fixed point, N decimals, "NaN" / "inf" / "-inf".
std::string fixed(double v, int decimals) {
    if (std::isnan(v)) return "NaN";
    if (std::isinf(v)) return v > 0 ? "inf" : "-inf";
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%.*f", decimals, v);
    return buf;
}

}  // namespace

double ColmapModel::mean_reprojection_error() const {
    double total = 0.0, count = 0.0;
    for (const auto &kv : points) {
        const double n = (double)kv.second.track.size();
        total += kv.second.error * n;
        count += n;
    }
    return count > 0.0 ? total / count : 0.0;
}

ColmapModel colmap_read(const std::string &dir) {
    namespace fs = std::filesystem;
    ColmapModel m;
    const fs::path d(dir);
    // cameras.txt (colmap.rs:70-111)
    for (const std::string &line : trimmed_lines(read_file((d / "cameras.txt").string()))) {
        if (line.empty() || line[0] == '#') continue;
        const auto tok = split_ws(line);
        if (tok.size() < 4) parse_fail("cameras.txt", "malformed line: " + line);
        ColmapCamera c;
        if (!parse_int(tok[0], c.id)) parse_fail("cameras.txt", "bad CAMERA_ID");
        if (!parse_int(tok[2], c.width)) parse_fail("cameras.txt", "bad WIDTH");
        if (!parse_int(tok[3], c.height)) parse_fail("cameras.txt", "bad HEIGHT");
        std::vector<double> params;
        for (size_t k = 4; k < tok.size(); ++k) {
            double v;
            if (!parse_float(tok[k], v)) parse_fail("cameras.txt", "bad PARAMS");
            params.push_back(v);
        }
        int model = -1;
        for (int k = 0; k < 6; ++k)
            if (tok[1] == kModelNames[k]) model = k;
        if (model < 0) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "unknown camera model: " + tok[1]);
        // CameraModel::from_name_and_params reads the model's parameter
        // count from the list (camera.rs:85-134); extra values are ignored.
        if ((int)params.size() < model_dof(model))
            parse_fail("cameras.txt", "too few PARAMS for " + tok[1]);
        c.model = model;
        for (int k = 0; k < model_dof(model); ++k) c.params[k] = params[k];
        m.cameras[c.id] = c;
    }
    // images.txt (colmap.rs:150-219): comment and empty lines are skipped
    // before the header / POINTS2D pairing.
    std::vector<std::string> lines;
    for (std::string &line : trimmed_lines(read_file((d / "images.txt").string())))
        if (!line.empty() && line[0] != '#') lines.push_back(std::move(line));
    for (size_t li = 0; li < lines.size();) {
        const std::string &header = lines[li++];
        const auto tok = split_ws(header);
        if (tok.size() < 10) parse_fail("images.txt", "malformed header: " + header);
        ColmapImage im;
        if (!parse_int(tok[0], im.id)) parse_fail("images.txt", "bad IMAGE_ID");
        for (int k = 0; k < 4; ++k)
            if (!parse_float(tok[1 + k], im.q[k])) parse_fail("images.txt", "bad quaternion");
        for (int k = 0; k < 3; ++k)
            if (!parse_float(tok[5 + k], im.t[k])) parse_fail("images.txt", "bad translation");
        if (!parse_int(tok[8], im.camera_id)) parse_fail("images.txt", "bad CAMERA_ID");
        im.name = tok[9];
        // Pose::from_quaternion_wxyz_translation normalises the quaternion
        // (UnitQuaternion::from_quaternion, pose.rs:74-80).
        // (Quaternion::norm sums the vector part first, then w.)
        const double nq = std::sqrt(im.q[1] * im.q[1] + im.q[2] * im.q[2] + im.q[3] * im.q[3] + im.q[0] * im.q[0]);
        for (double &x : im.q) x /= nq;
        if (li >= lines.size()) parse_fail("images.txt", "missing POINTS2D line");
        const auto pt = split_ws(lines[li++]);
        for (size_t k = 0; k + 3 <= pt.size(); k += 3) {
            float x, y;
            int64_t pid;
            if (!parse_float(pt[k], x)) parse_fail("images.txt", "bad point x");
            if (!parse_float(pt[k + 1], y)) parse_fail("images.txt", "bad point y");
            if (!parse_int(pt[k + 2], pid)) parse_fail("images.txt", "bad POINT3D_ID");
            im.keypoints.emplace_back(x, y);
            im.point3d_ids.push_back(pid < 0 ? -1 : pid);
        }
        m.images[im.id] = std::move(im);
    }
    // points3D.txt (colmap.rs:251-305)
    for (const std::string &line : trimmed_lines(read_file((d / "points3D.txt").string()))) {
        if (line.empty() || line[0] == '#') continue;
        const auto tok = split_ws(line);
        if (tok.size() < 8) parse_fail("points3D.txt", "malformed line: " + line);
        ColmapPoint p;
        if (!parse_int(tok[0], p.id)) parse_fail("points3D.txt", "bad POINT3D_ID");
        static const char *const kXyz[3] = {"bad X", "bad Y", "bad Z"};
        for (int k = 0; k < 3; ++k)
            if (!parse_float(tok[1 + k], p.xyz[k])) parse_fail("points3D.txt", kXyz[k]);
        static const char *const kRgb[3] = {"bad R", "bad G", "bad B"};
        for (int k = 0; k < 3; ++k)
            if (!parse_int(tok[4 + k], p.color[k])) parse_fail("points3D.txt", kRgb[k]);
        if (!parse_float(tok[7], p.error)) parse_fail("points3D.txt", "bad ERROR");
        for (size_t k = 8; k + 2 <= tok.size(); k += 2) {
            uint32_t a, b;
            if (!parse_int(tok[k], a)) parse_fail("points3D.txt", "bad TRACK IMAGE_ID");
            if (!parse_int(tok[k + 1], b)) parse_fail("points3D.txt", "bad TRACK POINT2D_IDX");
            p.track.emplace_back(a, b);
        }
        m.points[p.id] = std::move(p);
    }
    return m;
}

void colmap_write(const ColmapModel &m, const std::string &dir) {
    namespace fs = std::filesystem;
    std::error_code ec;
    fs::create_directories(dir, ec);
    if (ec) throw Error(SFMBA_ERR_INVALID_ARGUMENT, "cannot create " + dir + ": " + ec.message());
    const fs::path d(dir);
    {  // colmap.rs:43-67
        std::string out = "# Camera list with one line of data per camera:\n"
                          "#   CAMERA_ID, MODEL, WIDTH, HEIGHT, PARAMS[]\n";
        out += "# Number of cameras: " + std::to_string(m.cameras.size()) + "\n";
        for (const auto &kv : m.cameras) {
            const ColmapCamera &c = kv.second;
            out += std::to_string(c.id) + " " + kModelNames[c.model] + " " + std::to_string(c.width) + " " +
                   std::to_string(c.height) + " ";
            for (int k = 0; k < model_dof(c.model); ++k) {
                if (k) out += " ";
                out += fixed(c.params[k], 10);
            }
            out += "\n";
        }
        write_file((d / "cameras.txt").string(), out);
    }
    {  // colmap.rs:113-148
        size_t total = 0;
        for (const auto &kv : m.images) total += kv.second.keypoints.size();
        const double mean_obs = m.images.empty() ? 0.0 : (double)total / (double)m.images.size();
        std::string out = "# Image list with two lines of data per image:\n"
                          "#   IMAGE_ID, QW, QX, QY, QZ, TX, TY, TZ, CAMERA_ID, NAME\n"
                          "#   POINTS2D[] as (X, Y, POINT3D_ID)\n";
        out += "# Number of images: " + std::to_string(m.images.size()) +
               ", mean observations per image: " + fixed(mean_obs, 1) + "\n";
        for (const auto &kv : m.images) {
            const ColmapImage &im = kv.second;
            out += std::to_string(im.id);
            for (double q : im.q) out += " " + fixed(q, 10);
            for (double t : im.t) out += " " + fixed(t, 10);
            out += " " + std::to_string(im.camera_id) + " " + im.name + "\n";
            for (size_t k = 0; k < im.keypoints.size(); ++k) {
                if (k) out += " ";
                out += fixed(im.keypoints[k].first, 3) + " " + fixed(im.keypoints[k].second, 3) + " " +
                       std::to_string(im.point3d_ids[k] < 0 ? -1LL : (long long)im.point3d_ids[k]);
            }
            out += "\n";
        }
        write_file((d / "images.txt").string(), out);
    }
    {  // colmap.rs:221-249
        std::string out = "# 3D point list with one line of data per point:\n"
                          "#   POINT3D_ID, X, Y, Z, R, G, B, ERROR, TRACK[] as (IMAGE_ID, POINT2D_IDX)\n";
        out += "# Number of points: " + std::to_string(m.points.size()) + "\n";
        for (const auto &kv : m.points) {
            const ColmapPoint &p = kv.second;
            out += std::to_string(p.id) + " " + fixed(p.xyz[0], 10) + " " + fixed(p.xyz[1], 10) + " " +
                   fixed(p.xyz[2], 10) + " " + std::to_string(p.color[0]) + " " + std::to_string(p.color[1]) +
                   " " + std::to_string(p.color[2]) + " " + fixed(p.error, 6) + " ";
            for (size_t k = 0; k < p.track.size(); ++k) {
                if (k) out += " ";
                out += std::to_string(p.track[k].first) + " " + std::to_string(p.track[k].second);
            }
            out += "\n";
        }
        write_file((d / "points3D.txt").string(), out);
    }
}

}  // namespace sfmba
