// Support code for the reference sources compiled as the oracle: the TBB /
// Random shim state, a PFM reader standing in for the OIIO image loader
// (reference src/core/ImageFileLoader.cpp), and no-op image writers (the
// oracle reads Image::pixels directly; reference src/core/Image.cpp needs OIIO).
#include <core/Image.h>
#include <core/ImageFileLoader.h>
#include <math/Random.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace wfshim {
static int g_workers = 0;
static unsigned long long g_seed = 42;
static std::vector<std::mt19937> g_rngs;
static std::mutex g_mu;

int num_workers()
{
    if (g_workers <= 0) {
        unsigned hc = std::thread::hardware_concurrency();
        g_workers = hc ? (int)hc : 4;
        if (g_workers > 64) g_workers = 64;
    }
    return g_workers;
}
void set_num_workers(int n)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_workers = n > 64 ? 64 : n;
    g_rngs.clear();
}
void set_seed(unsigned long long seed)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_seed = seed;
    g_rngs.clear();
}
std::mt19937& worker_rng()
{
    if (g_rngs.empty()) {
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_rngs.empty()) {
            std::vector<std::mt19937> v;
            for (int w = 0; w < 64; ++w) {
                std::seed_seq sq{(unsigned)(g_seed & 0xFFFFFFFFu), (unsigned)(g_seed >> 32), (unsigned)w, 0x5eedu};
                v.emplace_back(sq);
            }
            g_rngs.swap(v);
        }
    }
    return g_rngs[worker_index()];
}
}  // namespace wfshim

bool loadImageRGB(const std::string& path, LoadedImageRGB& out, const std::string& label)
{
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        std::fprintf(stderr, "WARNING: Could not open %s: %s\n", label.c_str(), path.c_str());
        return false;
    }
    char magic[3] = {0};
    int w = 0, h = 0;
    float scale = 0.0f;
    bool ok = std::fscanf(f, "%2s %d %d %f", magic, &w, &h, &scale) == 4 && std::strcmp(magic, "PF") == 0 && w > 0 && h > 0;
    if (ok) {
        std::fgetc(f);
        std::vector<float> rows((size_t)w * h * 3);
        ok = std::fread(rows.data(), sizeof(float), rows.size(), f) == rows.size();
        if (ok) {
            out.width = w;
            out.height = h;
            out.isEightBitSource = false;
            out.pixels.resize(rows.size());
            for (int y = 0; y < h; ++y)  // PFM rows run bottom to top
                std::memcpy(&out.pixels[(size_t)y * w * 3], &rows[(size_t)(h - 1 - y) * w * 3], sizeof(float) * 3 * w);
        }
    }
    std::fclose(f);
    return ok;
}

void Image::write(const std::string&, bool) const {}
void Image::writePreview(const std::string&) const {}
