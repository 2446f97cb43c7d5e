// listlayout.cpp -- host construction of the fluid-list layout (see listlayout.h).
#include "listlayout.h"

#include <algorithm>
#include <array>

#include "common.cuh"

namespace mflbm {

bool build_list_layout(const int8_t *walls_h2, int nx, int ny, int nz, int iper, int jper, int kper, ListLayout &out,
                       std::string &why) {
    const int64_t h2x = nx + 4, h2xy = (int64_t)(nx + 4) * (ny + 4);
    const int64_t h1x = nx + 2, h1xy = (int64_t)(nx + 2) * (ny + 2);
    auto wall = [&](int i, int j, int k) { return walls_h2[(i + 1) + h2x * (j + 1) + h2xy * (k + 1)]; };
    // fluid index of every interior cell, -1 for solid
    std::vector<int32_t> fid((size_t)nx * ny * nz, -1);
    auto at = [&](int i, int j, int k) -> int32_t & { return fid[(size_t)(i - 1) + (size_t)nx * ((j - 1) + (size_t)ny * (k - 1))]; };
    out = ListLayout();
    out.slice.assign((size_t)nz + 1, 0);
    int64_t nf = 0;
    for (int k = 1; k <= nz; ++k) {
        out.slice[k - 1] = (int32_t)nf;
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i)
                if (wall(i, j, k) == 0) {
                    if (nf >= INT32_MAX) { why = "more than 2^31-1 fluid nodes"; return false; }
                    at(i, j, k) = (int32_t)nf++;
                    out.cell1.push_back((int32_t)(i + h1x * j + h1xy * k));
                }
    }
    out.slice[nz] = (int32_t)nf;
    out.nf = nf;
    if (nf == 0) { why = "no fluid nodes"; return false; }
    if ((int64_t)nx * ny * nz >= ((int64_t)1 << 31) || h1xy * (nz + 2) >= ((int64_t)1 << 31)) {
        why = "lattice too large for 32-bit cell indices";
        return false;
    }
    const int per[3] = {iper, jper, kper};
    const int n[3] = {nx, ny, nz};
    std::array<int64_t, 19> links{};
    // pass 1: count link slots per storage direction, check the ghost rule
    out.nb.assign((size_t)18 * nf, 0);
    for (int pass = 0; pass < 2; ++pass) {
        std::array<int64_t, 19> cnt{};
        int64_t x = 0;
        for (int k = 1; k <= nz; ++k)
            for (int j = 1; j <= ny; ++j)
                for (int i = 1; i <= nx; ++i) {
                    if (wall(i, j, k) != 0) continue;
                    for (int d = 1; d <= 18; ++d) {
                        int c[3] = {i + EX(d), j + EY(d), k + EZ(d)};
                        for (int a = 0; a < 3; ++a) {
                            if (c[a] >= 1 && c[a] <= n[a]) continue;
                            if (!per[a]) {
                                why = "a fluid node borders the ghost layer of a non-periodic direction";
                                return false;
                            }
                            c[a] = c[a] < 1 ? c[a] + n[a] : c[a] - n[a];
                        }
                        const int32_t y = at(c[0], c[1], c[2]);
                        int64_t slot;
                        if (y >= 0) {
                            slot = y;
                        } else {
                            const int qa = OPP(d);   // the solid node's slot opp(d) lives in array opp(d)
                            slot = nf + cnt[qa]++;
                            if (pass == 1) {
                                out.link.push_back(qa);
                                out.link.push_back((int32_t)slot);
                                out.link.push_back((int32_t)(c[0] + h1x * c[1] + h1xy * c[2]));
                            }
                        }
                        if (pass == 1) out.nb[(size_t)(d - 1) * nf + x] = (int32_t)slot;
                    }
                    ++x;
                }
        links = cnt;
    }
    int64_t maxl = 0, tot = 0;
    for (int q = 1; q <= 18; ++q) { maxl = std::max(maxl, links[q]); tot += links[q]; }
    out.nlink = tot;
    out.stride = (nf + maxl + 31) / 32 * 32;
    if (out.stride >= ((int64_t)1 << 31)) { why = "direction array exceeds 2^31 elements"; return false; }
    return true;
}

}  // namespace mflbm
