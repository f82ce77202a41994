// Test helper: runs lpm::amg_build on a stiffness given in the device
// block-CSR layout (binary files in a directory) and writes the hierarchy
// back as binary files, for tests/test_amg_setup.py.
//   amg_harness DIR AGG_SPACING
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include "amg.h"

template <typename T>
static std::vector<T> rd(const std::string &path, size_t count)
{
    std::vector<T> v(count);
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f || std::fread(v.data(), sizeof(T), count, f) != count) {
        std::fprintf(stderr, "cannot read %s\n", path.c_str());
        std::exit(2);
    }
    std::fclose(f);
    return v;
}

template <typename V>
static void wr(const std::string &path, const V &v)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    std::fwrite(v.data(), sizeof(v[0]), v.size(), f);
    std::fclose(f);
}

static void wr_bsr(FILE *f, const std::string &p, const lpm::Bsr &A)
{
    std::fprintf(f, " %d %d %d %d", A.nbr, A.nbc, A.R, A.C);
    wr(p + "_ptr.bin", A.ptr);
    wr(p + "_col.bin", A.col);
    wr(p + "_val.bin", A.val);
}

int main(int argc, char **argv)
{
    if (argc < 3)
        return 2;
    const std::string d(argv[1]);
    int n = 0;
    {
        FILE *f = std::fopen((d + "/n.txt").c_str(), "r");
        if (!f || std::fscanf(f, "%d", &n) != 1)
            return 2;
        std::fclose(f);
    }
    auto xyz = rd<double>(d + "/xyz.bin", 3 * (size_t)n);
    auto mask = rd<uint8_t>(d + "/mask.bin", n);
    auto rowoff = rd<long long>(d + "/rowoff.bin", (size_t)n + 1);
    auto npad = rd<int>(d + "/npad.bin", n);
    auto nconn = rd<int>(d + "/nconn.bin", n);
    auto cols = rd<int>(d + "/cols.bin", (size_t)rowoff[n]);
    auto val = rd<double>(d + "/val.bin", 9 * (size_t)rowoff[n]);
    lpm::AmgInput in;
    in.n = n;
    in.xyz = xyz.data();
    in.mask = mask.data();
    in.rowoff = rowoff.data();
    in.npad = npad.data();
    in.nconn = nconn.data();
    in.cols = cols.data();
    in.val = val.data();
    lpm::AmgOptions opt;
    opt.agg_spacing = std::atof(argv[2]);
    lpm::AmgHierarchy H;
    const auto t0 = std::chrono::steady_clock::now();
    const int L = lpm::amg_build(in, H, opt);
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::fprintf(stderr, "amg_build %.3f s\n", sec);
    FILE *f = std::fopen((d + "/levels.txt").c_str(), "w");
    std::fprintf(f, "%d %d\n", L, H.coarse_n);
    for (size_t l = 0; l < H.levels.size(); l++) {
        const lpm::AmgLevel &lv = H.levels[l];
        std::fprintf(f, "%d %d %.17g", lv.nblock, lv.bs, lv.omega);
        const std::string p = d + "/L" + std::to_string(l);
        wr_bsr(f, p + "_A", lv.A);
        wr_bsr(f, p + "_P", lv.P);
        wr_bsr(f, p + "_Pt", lv.Pt);
        std::fprintf(f, "\n");
        wr(p + "_Dinv.bin", lv.Dinv);
    }
    wr_bsr(f, d + "/coarse_A", H.coarse_A);
    std::fprintf(f, "\n");
    std::fclose(f);
    wr(d + "/coarse_chol.bin", H.coarse_chol);
    wr(d + "/coarse_inv.bin", H.coarse_inv);
    return L >= 0 ? 0 : 1;
}
