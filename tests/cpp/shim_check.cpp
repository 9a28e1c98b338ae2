// A C++ caller written against tiralib's entry points, built against the
// header shims in include/tira_gb300/ and linked to libtvgb.so.  It votes a
// small seeded 3D field through tira::cuda::tensorvote3, takes its
// eigenvalues through tira::cuda::evals3_symmetric and blurs a volume with
// tira::cuda::gaussian_filter3d, all with host pointers, and writes the raw
// results to the file named on the command line (checked by
// tests/test_gpu_shim.py against the CPU oracle).  With --host it only
// builds the neighbour tables and checks the negative-device rule, which
// needs no GPU (tests/test_shim_build.py).
#include <tira_gb300/tensorvote.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

static float lcg(uint64_t& s) {
    s = s * 6364136223846793005ULL + 1442695040888963407ULL;
    return float((s >> 40) & 0xFFFFFF) / float(0x1000000) * 2.0f - 1.0f;
}

// glm::vec2 stand-in: the reference passes the 3D sigmas as a glm::vec2.
struct sigma_pair {
    float x, y;
};

// Host-only part (no GPU needed): the neighbour tables in the reference's
// calling form, and the eigen launcher's answer to a negative device index.
static int host_part(const char* path) {
    std::vector<tira::Neighbor2D> nb2 = tira::cpu::build_neighbors2d(7, 2.0f, 0.5f, 2, 10, true, true);
    auto nb3 = tira::cpu::build_neighbors3d(7, sigma_pair{2.0f, 0.5f});
    const float m9[9] = {2, 0, 0, 0, 1, 0, 0, 0, 3};
    float* ev = tira::cuda::evals3_symmetric<float>(m9, 1, -1);   // the reference would use its CPU path
    const int32_t counts[3] = {int32_t(nb2.size()), int32_t(nb3.size()), ev == nullptr ? 1 : 0};
    FILE* f = std::fopen(path, "wb");
    if (!f) return 3;
    std::fwrite(counts, sizeof(int32_t), 3, f);
    std::fwrite(nb2.data(), sizeof(tira::Neighbor2D), nb2.size(), f);
    std::fwrite(nb3.data(), sizeof(tira::Neighbor3D), nb3.size(), f);
    std::fclose(f);
    delete[] ev;
    std::printf("host ok %zu %zu\n", nb2.size(), nb3.size());
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s [--host] <out.bin>\n", argv[0]);
        return 2;
    }
    if (std::string(argv[1]) == "--host") return argc > 2 ? host_part(argv[2]) : 2;
    const unsigned s0 = 6, s1 = 7, s2 = 8;
    const size_t n = size_t(s0) * s1 * s2;
    std::vector<float> in(9 * n), out(9 * n, 0.0f);
    uint64_t seed = 12345;
    for (size_t i = 0; i < n; ++i) {     // A A^T, symmetric positive semi-definite
        float A[9];
        for (float& a : A) a = lcg(seed);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c)
                in[9 * i + 3 * r + c] = A[3 * r] * A[3 * c] + A[3 * r + 1] * A[3 * c + 1] + A[3 * r + 2] * A[3 * c + 2];
    }
    tira::cuda::tensorvote3<float>(in.data(), out.data(), s0, s1, s2, 1.5f, 0.0f, 5, 1, 0, true, true, 20, false);
    float* ev = tira::cuda::evals3_symmetric<float>(out.data(), n, 0);
    std::vector<float> vol(12 * 13 * 14);
    for (float& v : vol) v = lcg(seed);
    unsigned ow, oh, od;
    float* blurred = tira::cuda::gaussian_filter3d<float>(vol.data(), 14, 13, 12, 1.0f, 1.0f, 1.0f, ow, oh, od);
    FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 3;
    std::fwrite(in.data(), sizeof(float), in.size(), f);
    std::fwrite(out.data(), sizeof(float), out.size(), f);
    std::fwrite(ev, sizeof(float), 3 * n, f);
    std::fwrite(vol.data(), sizeof(float), vol.size(), f);
    std::fwrite(blurred, sizeof(float), size_t(ow) * oh * od, f);
    std::fclose(f);
    delete[] ev;
    std::free(blurred);
    std::printf("ok %u %u %u\n", ow, oh, od);
    return 0;
}
