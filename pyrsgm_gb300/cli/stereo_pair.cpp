// stereo_pair.cpp -- headless stereo CLI over pyrsgm::StereoMatcher, without
// OpenCV (the reference's examples/stereo_pair.cpp:46-141 reads PNGs and
// writes colour maps with OpenCV; this one reads and writes PGM/PFM).
//
//   pyrsgm_stereo_pair left.pgm right.pgm out_prefix [num_disparities=128]
//                      [pyramid_levels=2] [bt|census] [--gt gt.pfm [--mask nocc.pgm] [--max-disp N]]
//
// Writes <out_prefix>_disp.pfm (float disparity, 0 = invalid, bottom-up
// little-endian PFM), <out_prefix>_disp.pgm (disparity * 255 / D) and
// <out_prefix>_conf.pgm (confidence * 255); prints the level geometry, the
// time per frame and, with --gt, the disparity metrics.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "pyrsgm/pyrsgm.h"
#include "pyrsgm/pyrsgm_io.h"

namespace {

struct Dev {
    void* p = nullptr;
    size_t pitch = 0;
    Dev(size_t width_bytes, int h)
    {
        if (cudaMallocPitch(&p, &pitch, width_bytes, (size_t)h) != cudaSuccess) throw std::runtime_error("cudaMallocPitch failed");
    }
    ~Dev() { cudaFree(p); }
};

bool read_pgm(const std::string& path, std::vector<unsigned char>& img, int& w, int& h)
{
    char err[256];
    if (pyrsgm_gb300_read_pgm(path.c_str(), nullptr, 0, &w, &h, err, sizeof err) != 0) {
        std::cerr << err << "\n";
        return false;
    }
    img.resize((size_t)w * h);
    if (pyrsgm_gb300_read_pgm(path.c_str(), img.data(), (size_t)w, &w, &h, err, sizeof err) != 0) {
        std::cerr << err << "\n";
        return false;
    }
    return true;
}

}  // namespace

int main(int argc, char** argv)
{
    std::vector<std::string> pos;
    std::string gt_path, mask_path;
    float max_disp = -1.0f;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--gt" && i + 1 < argc) gt_path = argv[++i];
        else if (a == "--mask" && i + 1 < argc) mask_path = argv[++i];
        else if (a == "--max-disp" && i + 1 < argc) max_disp = (float)std::atof(argv[++i]);
        else pos.push_back(a);
    }
    if (pos.size() < 3) {
        std::cerr << "usage: " << argv[0]
                  << " left.pgm right.pgm out_prefix [num_disparities=128] [pyramid_levels=2] [bt|census]"
                     " [--gt gt.pfm [--mask nocc.pgm] [--max-disp N]]\n";
        return 2;
    }
    std::vector<unsigned char> left, right;
    int w = 0, h = 0, w2 = 0, h2 = 0;
    if (!read_pgm(pos[0], left, w, h) || !read_pgm(pos[1], right, w2, h2)) return 1;
    if (w != w2 || h != h2) {
        std::cerr << "image sizes differ\n";
        return 1;
    }
    pyrsgm::Params params;
    params.num_disparities = pos.size() > 3 ? std::atoi(pos[3].c_str()) : 128;
    params.pyramid_levels = pos.size() > 4 ? std::atoi(pos[4].c_str()) : 2;
    if (pos.size() > 5 && pos[5] == "census") {
        params.cost_mode = pyrsgm::CostMode::Census;
        params.p1 = 8;
        params.p2 = 32;
    }
    const std::string prefix = pos[2];
    try {
        pyrsgm::StereoMatcher sgm(w, h, params);
        std::cout << "pyrsgm " << pyrsgm::version() << ": " << w << "x" << h << ", D=" << sgm.params().num_disparities
                  << ", levels=" << sgm.numLevels() - 1 << ", device memory " << sgm.deviceMemoryBytes() / (1024 * 1024)
                  << " MiB\n";
        for (int l = 0; l < sgm.numLevels(); ++l) {
            const pyrsgm::LevelInfo li = sgm.levelInfo(l);
            std::cout << "  level " << l << ": " << li.width << "x" << li.height << ", labels " << li.num_labels
                      << ", max disparity " << li.max_disparity << (li.refine ? " (refine)" : " (coarse)") << "\n";
        }
        Dev dl(w, h), dr(w, h), dd(w * sizeof(float), h), dc(w * sizeof(float), h);
        cudaMemcpy2D(dl.p, dl.pitch, left.data(), w, w, h, cudaMemcpyHostToDevice);
        cudaMemcpy2D(dr.p, dr.pitch, right.data(), w, w, h, cudaMemcpyHostToDevice);
        auto run = [&] {
            sgm.compute(static_cast<const uint8_t*>(dl.p), dl.pitch, static_cast<const uint8_t*>(dr.p), dr.pitch,
                        nullptr, 0, static_cast<float*>(dd.p), dd.pitch, static_cast<float*>(dc.p), dc.pitch);
        };
        run();   // warm-up
        if (cudaDeviceSynchronize() != cudaSuccess) throw std::runtime_error("CUDA error");
        const int runs = 10;
        const auto t0 = std::chrono::steady_clock::now();
        for (int i = 0; i < runs; ++i) run();
        if (cudaDeviceSynchronize() != cudaSuccess) throw std::runtime_error("CUDA error");
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count() / runs;
        std::cout << "  " << ms << " ms per frame (" << 1000.0 / ms << " fps)\n";

        std::vector<float> disp((size_t)w * h), conf((size_t)w * h);
        cudaMemcpy2D(disp.data(), w * sizeof(float), dd.p, dd.pitch, w * sizeof(float), h, cudaMemcpyDeviceToHost);
        cudaMemcpy2D(conf.data(), w * sizeof(float), dc.p, dc.pitch, w * sizeof(float), h, cudaMemcpyDeviceToHost);
        char err[256];
        if (pyrsgm_gb300_write_pfm((prefix + "_disp.pfm").c_str(), disp.data(), w, w, h, err, sizeof err) != 0) {
            std::cerr << err << "\n";
            return 1;
        }
        std::vector<unsigned char> d8((size_t)w * h), c8((size_t)w * h);
        const float sd = 255.0f / (float)params.num_disparities;
        for (size_t i = 0; i < d8.size(); ++i) {
            const float v = disp[i] > 0.0f ? disp[i] * sd + 0.5f : 0.0f;
            d8[i] = (unsigned char)(v > 255.0f ? 255.0f : v);
            const float c = conf[i] * 255.0f + 0.5f;
            c8[i] = (unsigned char)(c > 255.0f ? 255.0f : (c < 0.0f ? 0.0f : c));
        }
        if (pyrsgm_gb300_write_pgm((prefix + "_disp.pgm").c_str(), d8.data(), w, w, h, err, sizeof err) != 0 ||
            pyrsgm_gb300_write_pgm((prefix + "_conf.pgm").c_str(), c8.data(), w, w, h, err, sizeof err) != 0) {
            std::cerr << err << "\n";
            return 1;
        }
        std::cout << "  wrote " << prefix << "_disp.pfm / _disp.pgm / _conf.pgm\n";
        if (!gt_path.empty()) {
            int gw = 0, gh = 0;
            if (pyrsgm_gb300_read_pfm(gt_path.c_str(), nullptr, 0, &gw, &gh, err, sizeof err) != 0 || gw != w || gh != h) {
                std::cerr << "ground truth: " << (gw != w || gh != h ? std::string("size differs") : std::string(err)) << "\n";
                return 1;
            }
            std::vector<float> gt((size_t)w * h);
            pyrsgm_gb300_read_pfm(gt_path.c_str(), gt.data(), w, &gw, &gh, err, sizeof err);
            std::vector<unsigned char> mask;
            int mw = 0, mh = 0;
            if (!mask_path.empty() && (!read_pgm(mask_path, mask, mw, mh) || mw != w || mh != h)) {
                std::cerr << "mask: unreadable or size differs\n";
                return 1;
            }
            pyrsgm_gb300_metrics m;
            pyrsgm_gb300_evaluate(disp.data(), w, gt.data(), w, mask.empty() ? nullptr : mask.data(), w, w, h,
                                  max_disp > 0.0f ? max_disp : (float)params.num_disparities, &m);
            std::printf("  evaluated %d, density %.2f %%, avg err %.3f, rms %.3f, bad0.5 %.2f %%, bad1 %.2f %%, "
                        "bad2 %.2f %%, bad4 %.2f %%, bad1(all) %.2f %%, bad2(all) %.2f %%\n",
                        m.evaluated, m.density, m.avg_err, m.rms_err, m.bad05, m.bad1, m.bad2, m.bad4, m.bad1_all,
                        m.bad2_all);
        }
    } catch (const std::exception& e) {
        std::cerr << e.what() << "\n";
        return 1;
    }
    return 0;
}
