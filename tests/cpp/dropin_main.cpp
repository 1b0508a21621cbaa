// dropin_main.cpp -- a plugin-style program that advances a grid with the
// drop-in MMSP::gpu::update (tests only).
//
// Built against the reference's own headers (-DUSE_REFERENCE_GRID, where
// they exist) or against tests/cpp/mini_grid.hpp.  Raw little-endian values,
// cell-major, are read from IN and the result is written to OUT.
//
// usage: dropin_main ch|ch_f32|gg|gg_f32|sparse IN OUT STEPS n0 n1 n2 [fields]
#ifdef USE_REFERENCE_GRID
#include "MMSP.hpp"
#else
#include "mini_grid.hpp"
#endif
#include "MMSP.gpu.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

template <typename T> static bool read_raw(const char* f, std::vector<T>& v)
{
    FILE* p = std::fopen(f, "rb");
    if (!p) return false;
    size_t n = std::fread(&v[0], sizeof(T), v.size(), p);
    std::fclose(p);
    return n == v.size();
}
template <typename T> static bool write_raw(const char* f, const std::vector<T>& v)
{
    FILE* p = std::fopen(f, "wb");
    if (!p) return false;
    size_t n = std::fwrite(&v[0], sizeof(T), v.size(), p);
    std::fclose(p);
    return n == v.size();
}

// the plugin's update(), as a user of the reference writes it
namespace MMSP {
template <int dim, typename T> void update(grid<dim, T>& g, int steps)
{
    MMSP::gpu::update(g, steps, MMSP::gpu::cahn_hilliard(1.0, 1.0, 0.002));
}
template <int dim, typename T> void update(grid<dim, vector<T> >& g, int steps)
{
    MMSP::gpu::update(g, steps, MMSP::gpu::grain_growth_shipped(0.01));
}
template <int dim, typename T> void update(grid<dim, sparse<T> >& g, int steps)
{
    MMSP::gpu::update(g, steps, MMSP::gpu::sparse_grain_growth_shipped(0.01, 1.0e-8, 32));
}
}  // namespace MMSP

// Sparse grids as the plain list file: int32 dim, int32 extents, then per
// cell int32 count and count x (int32 index, float64 value).
static int sparse_case(const char* in, const char* out, int steps, int n0, int n1, int n2)
{
    MMSP::grid<3, MMSP::sparse<double> > g(0, 0, n0, 0, n1, 0, n2);
    FILE* p = std::fopen(in, "rb");
    if (!p) return 2;
    int hdr[4];
    bool ok = std::fread(hdr, sizeof(int), 4, p) == 4 && hdr[0] == 3;
    for (int i = 0; ok && i < nodes(g); i++) {
        int count = 0;
        ok = std::fread(&count, sizeof(int), 1, p) == 1;
        for (int h = 0; ok && h < count; h++) {
            int index = 0;
            double v = 0.0;
            ok = std::fread(&index, sizeof(int), 1, p) == 1 && std::fread(&v, sizeof(double), 1, p) == 1;
            if (ok) MMSP::set(g(i), index) = v;
        }
    }
    std::fclose(p);
    if (!ok) return 2;
    MMSP::update(g, steps);
    p = std::fopen(out, "wb");
    if (!p) return 3;
    std::fwrite(hdr, sizeof(int), 4, p);
    for (int i = 0; i < nodes(g); i++) {
        int count = length(g(i));
        std::fwrite(&count, sizeof(int), 1, p);
        for (int h = 0; h < count; h++) {
            int index = MMSP::index(g(i), h);
            double v = MMSP::value(g(i), h);
            std::fwrite(&index, sizeof(int), 1, p);
            std::fwrite(&v, sizeof(double), 1, p);
        }
    }
    std::fclose(p);
    return 0;
}

template <typename T> static int scalar_case(const char* in, const char* out, int steps, int n0, int n1, int n2)
{
    MMSP::grid<3, T> g(0, 0, n0, 0, n1, 0, n2);
    std::vector<T> v((size_t)n0 * n1 * n2);
    if (!read_raw(in, v)) return 2;
    for (int i = 0; i < nodes(g); i++) g(i) = v[i];
    MMSP::update(g, steps);
    for (int i = 0; i < nodes(g); i++) v[i] = g(i);
    return write_raw(out, v) ? 0 : 3;
}

template <typename T> static int vector_case(const char* in, const char* out, int steps, int n0, int n1, int n2, int N)
{
    MMSP::grid<3, MMSP::vector<T> > g(N, 0, n0, 0, n1, 0, n2);
    std::vector<T> v((size_t)n0 * n1 * n2 * N);
    if (!read_raw(in, v)) return 2;
    for (int i = 0; i < nodes(g); i++)
        for (int j = 0; j < N; j++) g(i)[j] = v[(size_t)i * N + j];
    MMSP::update(g, steps);
    for (int i = 0; i < nodes(g); i++)
        for (int j = 0; j < N; j++) v[(size_t)i * N + j] = g(i)[j];
    return write_raw(out, v) ? 0 : 3;
}

// MMSP.main.hpp's loop through MMSP::gpu::run: snapshots BASE.<step>.dat
// every `inc` steps, and the final values as raw data in OUT.
template <typename T> static int run_scalar(const char* in, const char* base, const char* out, int steps, int inc,
                                            int n0, int n1, int n2)
{
    MMSP::grid<3, T> g(0, 0, n0, 0, n1, 0, n2);
    std::vector<T> v((size_t)n0 * n1 * n2);
    if (!read_raw(in, v)) return 2;
    for (int i = 0; i < nodes(g); i++) g(i) = v[i];
    MMSP::gpu::run(g, 0, steps, inc, std::string(base) + ".", ".dat", MMSP::gpu::cahn_hilliard(1.0, 1.0, 0.002));
    for (int i = 0; i < nodes(g); i++) v[i] = g(i);
    return write_raw(out, v) ? 0 : 3;
}

template <typename T> static int run_vector(const char* in, const char* base, const char* out, int steps, int inc,
                                            int n0, int n1, int n2, int N)
{
    MMSP::grid<3, MMSP::vector<T> > g(N, 0, n0, 0, n1, 0, n2);
    std::vector<T> v((size_t)n0 * n1 * n2 * N);
    if (!read_raw(in, v)) return 2;
    for (int i = 0; i < nodes(g); i++)
        for (int j = 0; j < N; j++) g(i)[j] = v[(size_t)i * N + j];
    MMSP::gpu::run(g, 0, steps, inc, std::string(base) + ".", ".dat", MMSP::gpu::grain_growth_shipped(0.01));
    for (int i = 0; i < nodes(g); i++)
        for (int j = 0; j < N; j++) v[(size_t)i * N + j] = g(i)[j];
    return write_raw(out, v) ? 0 : 3;
}

int main(int argc, char* argv[])
{
    // usage: dropin_main run_ch|run_gg IN BASE OUT STEPS INC n0 n1 n2 [fields]
    if (argc >= 10 && (std::string(argv[1]) == "run_ch" || std::string(argv[1]) == "run_gg")) {
        int steps = std::atoi(argv[5]), inc = std::atoi(argv[6]);
        int n0 = std::atoi(argv[7]), n1 = std::atoi(argv[8]), n2 = std::atoi(argv[9]);
        if (std::string(argv[1]) == "run_ch") return run_scalar<double>(argv[2], argv[3], argv[4], steps, inc, n0, n1, n2);
        int N = argc > 10 ? std::atoi(argv[10]) : 2;
        return run_vector<double>(argv[2], argv[3], argv[4], steps, inc, n0, n1, n2, N);
    }
    if (argc < 8) {
        std::fprintf(stderr, "usage: dropin_main ch|ch_f32|gg|gg_f32 IN OUT STEPS n0 n1 n2 [fields]\n");
        return 1;
    }
    std::string mode = argv[1];
    int steps = std::atoi(argv[4]), n0 = std::atoi(argv[5]), n1 = std::atoi(argv[6]), n2 = std::atoi(argv[7]);
    int N = argc > 8 ? std::atoi(argv[8]) : 2;
    if (mode == "ch") return scalar_case<double>(argv[2], argv[3], steps, n0, n1, n2);
    if (mode == "ch_f32") return scalar_case<float>(argv[2], argv[3], steps, n0, n1, n2);
    if (mode == "gg") return vector_case<double>(argv[2], argv[3], steps, n0, n1, n2, N);
    if (mode == "gg_f32") return vector_case<float>(argv[2], argv[3], steps, n0, n1, n2, N);
    if (mode == "sparse") return sparse_case(argv[2], argv[3], steps, n0, n1, n2);
    return 1;
}
