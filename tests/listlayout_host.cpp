// listlayout_host.cpp -- the fluid-list layout builder (mf-lbm_gb300/csrc/listlayout.cpp)
// built for the host, with a decoder of the warp-compressed neighbour table that follows
// the odd-step kernel (k_sp_list_odd8) lane by lane, the warp ballot emulated: the CPU test
// checks that every decoded slot equals the 32-bit table's.
#include <cstdint>
#include <string>
#include <vector>

#include "../mf-lbm_gb300/csrc/listlayout.cpp"

extern "C" {

// Builds the layout of a halo-2 wall array and decodes the warp table.  Returns the number
// of mismatching (node, direction) entries, or -1 when the layout cannot be built; *nf,
// *nwide (wide warp-directions) and *nlink report the layout.
int64_t llh_check(const int8_t *walls, int nx, int ny, int nz, int iper, int jper, int kper, int64_t *nf,
                  int64_t *nwide, int64_t *nlink) {
    mflbm::ListLayout ll;
    std::string why;
    if (!mflbm::build_list_layout(walls, nx, ny, nz, iper, jper, kper, ll, why)) return -1;
    mflbm::build_warp_table(ll);
    *nf = ll.nf;
    *nlink = ll.nlink;
    *nwide = (int64_t)ll.side.size() / 32;
    int64_t bad = 0;
    const int64_t n = ll.nf;
    for (int64_t w = 0; w * 32 < n; ++w) {
        for (int d = 0; d < 18; ++d) {
            const int32_t fb = ll.hdr[(size_t)2 * (18 * w + d)], lb = ll.hdr[(size_t)2 * (18 * w + d) + 1];
            // ballot of the lanes holding a link
            uint32_t lm = 0;
            for (int lane = 0; lane < 32; ++lane) {
                const int64_t t = 32 * w + lane;
                if (t < n && ll.off8[(size_t)d * n + t] == 255) lm |= 1u << lane;
            }
            for (int lane = 0; lane < 32; ++lane) {
                const int64_t t = 32 * w + lane;
                if (t >= n) continue;
                const int c = ll.off8[(size_t)d * n + t];
                int64_t slot;
                if (lb < 0) slot = ll.side[(size_t)fb + lane];
                else if (c == 255) slot = lb + __builtin_popcount(lm & ((1u << lane) - 1u));
                else slot = t + fb + c;
                if (slot != ll.nb[(size_t)d * n + t]) ++bad;
            }
        }
    }
    return bad;
}
}
