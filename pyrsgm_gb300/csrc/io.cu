// io.cu -- PFM / PGM files and disparity metrics (host code only).  The
// reference keeps these in its OpenCV-based benchmark and example
// (bench/middlebury.h:22-120, examples/stereo_pair.cpp:37-44); here they are
// plain C++ behind the C ABI of pyrsgm_io.h.
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "pyrsgm/pyrsgm_io.h"

namespace {

int fail(char* err, size_t len, const std::string& msg)
{
    if (err && len) {
        std::snprintf(err, len, "%s", msg.c_str());
    }
    return -1;
}

// Next whitespace-separated header token of a PNM/PFM file, skipping
// '#' comments; consumes exactly one whitespace byte after the token.
bool header_token(std::istream& f, std::string& tok)
{
    tok.clear();
    int c = f.get();
    for (;;) {
        while (c != EOF && std::isspace(c)) c = f.get();
        if (c == '#') {
            while (c != EOF && c != '\n') c = f.get();
            continue;
        }
        break;
    }
    while (c != EOF && !std::isspace(c)) {
        tok.push_back((char)c);
        c = f.get();
    }
    return !tok.empty();
}

bool host_little_endian()
{
    const uint32_t one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

uint32_t bswap32(uint32_t u) { return (u << 24) | ((u & 0xff00u) << 8) | ((u >> 8) & 0xff00u) | (u >> 24); }

}  // namespace

extern "C" {

int pyrsgm_gb300_read_pfm(const char* path, float* data, size_t pitch, int* width, int* height, char* err,
                          size_t err_len)
{
    if (!path || !width || !height) return fail(err, err_len, "null argument");
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(err, err_len, std::string("cannot open ") + path);
    std::string magic, sw, sh, ss;
    if (!header_token(f, magic) || magic != "Pf")
        return fail(err, err_len, std::string(path) + ": not a grayscale PFM (Pf)");
    if (!header_token(f, sw) || !header_token(f, sh) || !header_token(f, ss))
        return fail(err, err_len, std::string(path) + ": truncated PFM header");
    const int w = std::atoi(sw.c_str()), h = std::atoi(sh.c_str());
    const double scale = std::atof(ss.c_str());
    if (w <= 0 || h <= 0 || scale == 0.0) return fail(err, err_len, std::string(path) + ": bad PFM header");
    *width = w;
    *height = h;
    if (!data) return 0;
    if (pitch < (size_t)w) return fail(err, err_len, "pitch smaller than the width");
    const bool swap = (scale < 0.0) != host_little_endian();   // scale < 0: little-endian data
    std::vector<float> row((size_t)w);
    for (int y = h - 1; y >= 0; --y) {   // bottom row first
        f.read(reinterpret_cast<char*>(row.data()), (std::streamsize)(w * sizeof(float)));
        if (!f) return fail(err, err_len, std::string(path) + ": truncated PFM data");
        float* dst = data + (size_t)y * pitch;
        for (int x = 0; x < w; ++x) {
            float v = row[x];
            if (swap) {
                uint32_t u;
                std::memcpy(&u, &v, 4);
                u = bswap32(u);
                std::memcpy(&v, &u, 4);
            }
            dst[x] = v;
        }
    }
    return 0;
}

int pyrsgm_gb300_write_pfm(const char* path, const float* data, size_t pitch, int width, int height, char* err,
                           size_t err_len)
{
    if (!path || !data || width <= 0 || height <= 0 || pitch < (size_t)width)
        return fail(err, err_len, "bad arguments");
    std::ofstream f(path, std::ios::binary);
    if (!f) return fail(err, err_len, std::string("cannot create ") + path);
    f << "Pf\n" << width << " " << height << "\n-1.0\n";
    std::vector<float> row((size_t)width);
    const bool swap = !host_little_endian();
    for (int y = height - 1; y >= 0; --y) {
        const float* src = data + (size_t)y * pitch;
        for (int x = 0; x < width; ++x) {
            float v = src[x];
            if (swap) {
                uint32_t u;
                std::memcpy(&u, &v, 4);
                u = bswap32(u);
                std::memcpy(&v, &u, 4);
            }
            row[x] = v;
        }
        f.write(reinterpret_cast<const char*>(row.data()), (std::streamsize)(width * sizeof(float)));
    }
    return f ? 0 : fail(err, err_len, std::string("write failed: ") + path);
}

int pyrsgm_gb300_read_pgm(const char* path, unsigned char* data, size_t pitch, int* width, int* height, char* err,
                          size_t err_len)
{
    if (!path || !width || !height) return fail(err, err_len, "null argument");
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(err, err_len, std::string("cannot open ") + path);
    std::string magic, sw, sh, sm;
    if (!header_token(f, magic) || magic != "P5")
        return fail(err, err_len, std::string(path) + ": not a binary PGM (P5)");
    if (!header_token(f, sw) || !header_token(f, sh) || !header_token(f, sm))
        return fail(err, err_len, std::string(path) + ": truncated PGM header");
    const int w = std::atoi(sw.c_str()), h = std::atoi(sh.c_str()), maxval = std::atoi(sm.c_str());
    if (w <= 0 || h <= 0 || maxval <= 0 || maxval > 255)
        return fail(err, err_len, std::string(path) + ": unsupported PGM (8-bit only)");
    *width = w;
    *height = h;
    if (!data) return 0;
    if (pitch < (size_t)w) return fail(err, err_len, "pitch smaller than the width");
    for (int y = 0; y < h; ++y) {
        f.read(reinterpret_cast<char*>(data + (size_t)y * pitch), w);
        if (!f) return fail(err, err_len, std::string(path) + ": truncated PGM data");
    }
    return 0;
}

int pyrsgm_gb300_write_pgm(const char* path, const unsigned char* data, size_t pitch, int width, int height,
                           char* err, size_t err_len)
{
    if (!path || !data || width <= 0 || height <= 0 || pitch < (size_t)width)
        return fail(err, err_len, "bad arguments");
    std::ofstream f(path, std::ios::binary);
    if (!f) return fail(err, err_len, std::string("cannot create ") + path);
    f << "P5\n" << width << " " << height << "\n255\n";
    for (int y = 0; y < height; ++y) f.write(reinterpret_cast<const char*>(data + (size_t)y * pitch), width);
    return f ? 0 : fail(err, err_len, std::string("write failed: ") + path);
}

int pyrsgm_gb300_read_ndisp(const char* path)
{
    if (!path) return 0;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line))
        if (line.compare(0, 6, "ndisp=") == 0) return std::atoi(line.c_str() + 6);
    return 0;
}

int pyrsgm_gb300_evaluate(const float* disp, size_t disp_pitch, const float* gt, size_t gt_pitch,
                          const unsigned char* mask, size_t mask_pitch, int width, int height, float max_disp,
                          pyrsgm_gb300_metrics* out)
{
    if (!disp || !gt || !out || width <= 0 || height <= 0) return -1;
    pyrsgm_gb300_metrics m{};
    double sum = 0.0, sq = 0.0;
    long long over05 = 0, over1 = 0, over2 = 0, over4 = 0;
    for (int y = 0; y < height; ++y) {
        const float* d = disp + (size_t)y * disp_pitch;
        const float* g = gt + (size_t)y * gt_pitch;
        const unsigned char* mk = mask ? mask + (size_t)y * mask_pitch : nullptr;
        for (int x = 0; x < width; ++x) {
            const float t = g[x];
            if (!std::isfinite(t) || t <= 0.0f || t > max_disp) continue;   // unknown ground truth
            if (mk && mk[x] != 255) continue;
            ++m.evaluated;
            if (!(d[x] > 0.0f)) continue;   // invalid estimate (also NaN)
            ++m.valid;
            const double e = std::fabs((double)d[x] - (double)t);
            sum += e;
            sq += e * e;
            over05 += e > 0.5;
            over1 += e > 1.0;
            over2 += e > 2.0;
            over4 += e > 4.0;
        }
    }
    if (m.valid) {
        m.avg_err = sum / m.valid;
        m.rms_err = std::sqrt(sq / m.valid);
        m.bad05 = 100.0 * over05 / m.valid;
        m.bad1 = 100.0 * over1 / m.valid;
        m.bad2 = 100.0 * over2 / m.valid;
        m.bad4 = 100.0 * over4 / m.valid;
    }
    if (m.evaluated) {
        const long long missing = m.evaluated - m.valid;
        m.density = 100.0 * m.valid / m.evaluated;
        m.invalid = 100.0 - m.density;
        m.bad1_all = 100.0 * (over1 + missing) / m.evaluated;
        m.bad2_all = 100.0 * (over2 + missing) / m.evaluated;
    }
    *out = m;
    return 0;
}

}  // extern "C"
