// mplist_host.cpp -- the multiphase fluid-list layout builder (mf-lbm_gb300/csrc/listlayout.cpp)
// built for the host, with checks of every index it hands to the device: neighbour slots and
// map entries inside the direction arrays, one slot per (solid cell, array) for the links,
// boundary-plane cells all resolved to a slot, and the neighbour of a fluid node in a
// boundary plane equal to the slot a boundary condition addresses for that cell.
#include <algorithm>
#include <cstdint>
#include <set>
#include <string>
#include <vector>

#include "../mf-lbm_gb300/csrc/listlayout.cpp"

static mflbm::MpListLayout g_layout;

extern "C" {

// Builds a layout and keeps it for mph_get.  info: nf, nplane, nlink, stride, spare, map
// size, nwrap.  Returns -1 when the layout cannot be built.
int64_t mph_build(const int8_t *walls, int nx, int ny, int nz, int jper, int kper, const int *planes, int nplanes,
                  const int *ghost_planes, int nghost, int64_t *info) {
    std::vector<int> pl(planes, planes + nplanes), gp(ghost_planes, ghost_planes + nghost);
    std::string why;
    if (!mflbm::build_mp_list_layout(walls, nx, ny, nz, jper, kper, pl, gp, g_layout, why)) return -1;
    info[0] = g_layout.nf;
    info[1] = g_layout.nplane;
    info[2] = g_layout.nlink;
    info[3] = g_layout.stride;
    info[4] = g_layout.spare;
    info[5] = (int64_t)g_layout.map.size();
    info[6] = g_layout.nwrap;
    return 0;
}

// Copies the tables of the last mph_build (sizes from its info).
void mph_get(int32_t *map, int32_t *nb, int32_t *link, int32_t *cell1, int32_t *wrap) {
    std::copy(g_layout.map.begin(), g_layout.map.end(), map);
    std::copy(g_layout.nb.begin(), g_layout.nb.end(), nb);
    std::copy(g_layout.link.begin(), g_layout.link.end(), link);
    std::copy(g_layout.cell1.begin(), g_layout.cell1.end(), cell1);
    std::copy(g_layout.wrap.begin(), g_layout.wrap.end(), wrap);
}

// Returns the number of failed checks, or -1 when the layout cannot be built.
int64_t mph_check(const int8_t *walls, int nx, int ny, int nz, int jper, int kper, int open_z, int z_pp, int64_t *nf,
                  int64_t *nplane, int64_t *nlink, int64_t *stride) {
    std::vector<int> planes, ghost_planes;
    if (open_z)
        for (int k : {0, 1, 2, nz - 1, nz, nz + 1}) planes.push_back(k);
    if (z_pp > 0)
        for (int dz = -1; dz <= 1; ++dz) {
            planes.push_back(z_pp + dz);
            ghost_planes.push_back(z_pp + dz);
        }
    mflbm::MpListLayout ml;
    std::string why;
    if (!mflbm::build_mp_list_layout(walls, nx, ny, nz, jper, kper, planes, ghost_planes, ml, why)) return -1;
    *nf = ml.nf;
    *nplane = ml.nplane;
    *nlink = ml.nlink;
    *stride = ml.stride;
    int64_t bad = 0;
    const int64_t h1x = nx + 2, h1xy = (int64_t)(nx + 2) * (ny + 2);
    auto resolve = [&](int64_t m) -> int64_t { return m >= 0 ? m : (m <= -2 ? -m - 2 : -1); };
    for (size_t t = 0; t < ml.nb.size(); ++t)
        if (ml.nb[t] < 0 || ml.nb[t] >= ml.stride) ++bad;
    for (int32_t m : ml.map) {
        const int64_t r = resolve(m);
        if (m != -1 && (r < 0 || r >= ml.spare)) ++bad;
    }
    if (ml.spare >= ml.stride) ++bad;
    std::set<std::pair<int, int32_t>> seen;
    for (int64_t l = 0; l < ml.nlink; ++l) {
        const int q = ml.link[3 * l];
        const int32_t slot = ml.link[3 * l + 1];
        if (q < 1 || q > 18 || slot <= ml.spare || slot >= ml.stride) ++bad;
        if (!seen.insert({q, slot}).second) ++bad;
    }
    for (int k : planes) {
        if (k < 0 || k > nz + 1) continue;
        for (int j = 0; j <= ny + 1; ++j)
            for (int i = 0; i <= nx + 1; ++i)
                if (resolve(ml.map[(size_t)(i + h1x * j + h1xy * k)]) < 0) ++bad;
    }
    // the porous-plate ghost exchange: private ghost slots, images inside the owned range
    for (int64_t w = 0; w < ml.nwrap; ++w) {
        const int32_t *e = &ml.wrap[(size_t)(4 * w)];
        if (e[0] < ml.nf || e[0] >= ml.spare || e[2] < ml.nf || e[2] >= ml.spare) ++bad;
        if (e[1] < 0 || e[1] >= ml.spare || e[3] < 0 || e[3] >= ml.spare) ++bad;
    }
    if (jper && z_pp > 0 && ml.nwrap != 3 * (int64_t)nx) ++bad;
    // a fluid node's neighbour inside a boundary plane: the table's slot is the map's slot
    std::vector<char> inplane((size_t)nz + 2, 0);
    for (int k : planes)
        if (k >= 0 && k <= nz + 1) inplane[(size_t)k] = 1;
    for (int64_t x = 0; x < ml.nf; ++x) {
        const int64_t c = ml.cell1[(size_t)x];
        const int i = (int)(c % h1x), j = (int)((c / h1x) % (ny + 2)), k = (int)(c / h1xy);
        if (resolve(ml.map[(size_t)c]) != x) ++bad;
        for (int d = 1; d <= 18; ++d) {
            const int ci = i + mflbm::EX(d), cj = j + mflbm::EY(d), ck = k + mflbm::EZ(d);
            if (!inplane[(size_t)ck]) continue;
            const int64_t m = resolve(ml.map[(size_t)(ci + h1x * cj + h1xy * ck)]);
            if (m != ml.nb[(size_t)(d - 1) * ml.nf + x]) ++bad;
        }
    }
    return bad;
}
}
