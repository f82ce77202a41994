// Host-side choice of the bonds that break in one brittle pass
// (updateBrittleDamage, src/constitutive.c:1437-1527), called by the damage
// stage after the candidate kernel has collected the bonds.
// Input: candidate bonds b = j * n + i (slot j of particle i, in any order)
// with their bond strains.  They are put into the reference's scan order
// (particle, then slot); when there are more than nbreak, the reference's
// shell sort (ascending strain, gaps k/2, k/4, ..., 1) orders them and the
// last nbreak (largest strains) are chosen.  Returns the chosen bonds in the
// order the reference breaks and logs them.
#pragma once
#include <algorithm>
#include <numeric>
#include <vector>

namespace lpm {

inline std::vector<int> brittle_select(const std::vector<int> &bonds, const std::vector<double> &strain, int n,
                                       int nbreak)
{
    const int k = (int)bonds.size();
    std::vector<int> idx(k);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](int x, int y) {
        const int ix = bonds[x] % n, iy = bonds[y] % n;
        return ix != iy ? ix < iy : bonds[x] / n < bonds[y] / n;
    });
    std::vector<int> bi(k);
    std::vector<double> bs(k);
    for (int q = 0; q < k; q++) {
        bi[q] = bonds[idx[q]];
        bs[q] = strain[idx[q]];
    }
    int first = 0;
    if (k > nbreak) {
        for (int r = k / 2; r >= 1; r = r / 2)
            for (int i = r; i < k; ++i) {
                const int tb = bi[i];
                const double ts = bs[i];
                int j = i - r;
                while (j >= 0 && bs[j] > ts) {
                    bs[j + r] = bs[j];
                    bi[j + r] = bi[j];
                    j = j - r;
                }
                bs[j + r] = ts;
                bi[j + r] = tb;
            }
        first = k - nbreak;
    }
    return std::vector<int>(bi.begin() + first, bi.end());
}

}  // namespace lpm
