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

bool build_mp_list_layout(const int8_t *walls_h2, int nx, int ny, int nz, int jper, int kper,
                          const std::vector<int> &planes, const std::vector<int> &ghost_planes, MpListLayout &out,
                          std::string &why) {
    const int64_t h2x = nx + 4, h2xy = (int64_t)(nx + 4) * (ny + 4);
    const int64_t h1x = nx + 2, h1xy = (int64_t)(nx + 2) * (ny + 2);
    const int64_t n1 = h1xy * (nz + 2);
    if (n1 >= ((int64_t)1 << 31) - 64) { why = "lattice too large for 32-bit slot maps"; return false; }
    auto wall = [&](int i, int j, int k) { return walls_h2[(i + 1) + h2x * (j + 1) + h2xy * (k + 1)]; };
    auto h1 = [&](int i, int j, int k) { return (int64_t)i + h1x * j + h1xy * k; };
    out = MpListLayout();
    out.map.assign((size_t)n1, -1);
    out.slice.assign((size_t)nz + 1, 0);
    int64_t nf = 0;
    for (int k = 1; k <= nz; ++k) {
        out.slice[k - 1] = (int32_t)nf;
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i)
                if (wall(i, j, k) == 0) {
                    out.map[(size_t)h1(i, j, k)] = (int32_t)nf++;
                    out.cell1.push_back((int32_t)h1(i, j, k));
                }
    }
    out.slice[nz] = (int32_t)nf;
    out.nf = nf;
    if (nf == 0) { why = "no fluid nodes"; return false; }
    // the periodic image the halo exchange copies into a ghost cell (Mpi.F90 for one rank:
    // y faces over i in [1, nx], k in [1, nz]; z faces over i in [1, nx], j in [1, ny]; the
    // x-aligned edges when y and z are both periodic); false when the cell is not such a ghost
    auto image = [&](int i, int j, int k, int &ii, int &jj, int &kk) {
        if (i < 1 || i > nx) return false;
        const bool gy = j < 1 || j > ny, gz = k < 1 || k > nz;
        if (!gy && !gz) return false;
        if (gy && !jper) return false;
        if (gz && !kper) return false;
        ii = i;
        jj = gy ? (j < 1 ? j + ny : j - ny) : j;
        kk = gz ? (k < 1 ? k + nz : k - nz) : k;
        return true;
    };
    // private slots of the boundary planes (and of the y ghosts of the ghost planes)
    int64_t next = nf;
    std::vector<char> inplane((size_t)nz + 2, 0), ownghost((size_t)nz + 2, 0);
    for (int k : planes)
        if (k >= 0 && k <= nz + 1) inplane[(size_t)k] = 1;
    for (int k : ghost_planes) {
        if (!jper) continue;
        if (k < 1 || k > nz) { why = "porous-plate planes outside [1, nz]"; return false; }
        inplane[(size_t)k] = 1;
        ownghost[(size_t)k] = 1;
    }
    auto private_ghost = [&](int i, int j, int k) {
        return ownghost[(size_t)k] && i >= 1 && i <= nx && (j == 0 || j == ny + 1);
    };
    for (int k = 0; k <= nz + 1; ++k) {
        if (!inplane[(size_t)k]) continue;
        for (int j = 0; j <= ny + 1; ++j)
            for (int i = 0; i <= nx + 1; ++i) {
                int ii, jj, kk;
                if (out.map[(size_t)h1(i, j, k)] >= 0) continue;
                if (image(i, j, k, ii, jj, kk) && !private_ghost(i, j, k)) continue;
                out.map[(size_t)h1(i, j, k)] = (int32_t)next++;
            }
    }
    out.nplane = next - nf;
    out.spare = next++;
    // images of the periodic ghosts, after every owned slot is known
    for (int k = 0; k <= nz + 1; ++k)
        for (int j = 0; j <= ny + 1; ++j)
            for (int i = 0; i <= nx + 1; ++i) {
                int ii, jj, kk;
                if (private_ghost(i, j, k) || !image(i, j, k, ii, jj, kk)) continue;
                const int32_t m = out.map[(size_t)h1(ii, jj, kk)];
                if (m >= 0) out.map[(size_t)h1(i, j, k)] = -m - 2;
            }
    // the exchange of the private y ghosts: {ghost 0, image ny, ghost ny + 1, image 1}
    for (int k = 1; k <= nz; ++k) {
        if (!ownghost[(size_t)k]) continue;
        for (int i = 1; i <= nx; ++i) {
            const int32_t s[4] = {out.map[(size_t)h1(i, 0, k)], out.map[(size_t)h1(i, ny, k)],
                                  out.map[(size_t)h1(i, ny + 1, k)], out.map[(size_t)h1(i, 1, k)]};
            for (int32_t v : s)
                if (v < 0) { why = "a porous-plate plane cell without a slot"; return false; }
            out.wrap.insert(out.wrap.end(), s, s + 4);
            ++out.nwrap;
        }
    }
    const int64_t base = next;
    // neighbour table and the link slots of solid cells outside the boundary planes
    std::array<int64_t, 19> cnt{};
    out.nb.assign((size_t)18 * nf, 0);
    for (int64_t x = 0; x < nf; ++x) {
        const int64_t c = out.cell1[(size_t)x];
        const int i = (int)(c % h1x), j = (int)((c / h1x) % (ny + 2)), k = (int)(c / h1xy);
        for (int d = 1; d <= 18; ++d) {
            int ci = i + EX(d), cj = j + EY(d), ck = k + EZ(d);
            int ii, jj, kk;
            if (ci < 0 || ci > nx + 1 || cj < 0 || cj > ny + 1 || ck < 0 || ck > nz + 1) {
                why = "a neighbour outside the halo-1 box";
                return false;
            }
            if (!private_ghost(ci, cj, ck) && image(ci, cj, ck, ii, jj, kk)) { ci = ii; cj = jj; ck = kk; }
            const int32_t m = out.map[(size_t)h1(ci, cj, ck)];
            int64_t slot;
            if (m >= 0) {
                slot = m;
            } else {
                const int qa = OPP(d);   // the solid cell's slot opp(d), in array opp(d)
                slot = base + cnt[qa]++;
                out.link.push_back(qa);
                out.link.push_back((int32_t)slot);
                out.link.push_back((int32_t)h1(ci, cj, ck));
            }
            out.nb[(size_t)(d - 1) * nf + x] = (int32_t)slot;
        }
    }
    int64_t maxl = 0, tot = 0;
    for (int q = 1; q <= 18; ++q) { maxl = std::max(maxl, cnt[q]); tot += cnt[q]; }
    out.nlink = tot;
    out.stride = (base + maxl + 31) / 32 * 32;
    if (out.stride >= ((int64_t)1 << 31)) { why = "direction array exceeds 2^31 elements"; return false; }
    return true;
}

}  // namespace mflbm
