// listlayout.h -- the fluid-list storage of singlephase samples (host construction).
//
// The dense layout stores every lattice cell; at porosity 0.2-0.3 most 32-byte sectors
// of a PDF plane mix fluid slots with solid ones, so the sweep moves nearly the whole
// plane each step.  The fluid-list layout stores, per direction q, only:
//   [0, nf)          the fluid nodes, in cell order (k, j, i)
//   [nf, nf+links_q) one slot per bounce-back link whose storage is this direction
// and an 18-entry neighbour table per fluid node.  The AA-pattern update stays exactly
// the reference's (kernel_odd / kernel_even, singlephase_3D/0.src/Kernel.F90:5-400):
//   odd : ft_q <- A_q[nb[opp q][x]]        ... A_opp(q)[nb[q][x]] <- ft_q
//   even: ft_q <- A_opp(q)[x]              ... A_q[x] <- ft_q
// nb[d][x] is the fluid index of x + e_d (periodic directions wrap), or, when x + e_d is
// solid, the link slot that plays the solid node's slot opp(d): the population x pushes
// into the wall at an odd step comes back from it at the next odd step, the reference's
// full-way bounce-back through untouched solid slots.  A periodic wrap through the
// neighbour table equals the reference's self-exchange of halo faces and edges
// (Mpi.F90 pack/unpack), which D3Q19 (no corner directions) reduces to a plain wrap.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace mflbm {

struct ListLayout {
    int64_t nf = 0;                 // fluid nodes
    int64_t stride = 0;             // elements per direction array (nf + max links, padded)
    int64_t nlink = 0;              // bounce-back link slots over all directions
    std::vector<int32_t> nb;        // [18][nf], direction d = 1..18 at row d-1
    std::vector<int32_t> cell1;     // halo-1 Fortran index of every fluid node
    std::vector<int32_t> link;      // [nlink][3]: direction array q, slot index, halo-1 index of the solid cell
    std::vector<int32_t> slice;     // [nz+1]: first fluid index of every z slice
};


// Builds the layout for one sample from the halo-2 wall array (Fortran order, int8,
// 1 = solid).  Returns false with a reason when a fluid node has a neighbour in the
// ghost layer of a non-periodic direction (open boundaries need the dense layout).
bool build_list_layout(const int8_t *walls_h2, int nx, int ny, int nz, int iper, int jper, int kper, ListLayout &out,
                       std::string &why);

// The multiphase fluid-list layout (f and g each as 19 direction arrays of `stride` slots):
//   [0, nf)                     fluid nodes, in cell order (k, j, i)
//   [nf, nf + nplane)           private slots of the boundary planes: every solid or ghost
//                               cell of the planes the inlet, outlet and porous-plate
//                               conditions read or write (k = 0, 1, 2, nz-1, nz, nz+1 when z
//                               is open; z_pp - 1 .. z_pp + 1 for a porous plate), one slot
//                               per cell, the same index in every direction array
//                               (for the porous plate's planes with y periodic, the y ghosts
//                               too: see `wrap` below)
//   nf + nplane                 a spare slot for cells that have none (never read for a value)
//   [nf + nplane + 1, ...)      one slot per bounce-back link into a solid cell outside the
//                               boundary planes, in the array that holds the solid cell's slot
// nb[d][x] is the slot of x + e_d, resolved as the dense layout reads it: a neighbour in a
// periodic face, edge or corner that the reference's halo exchange fills is its periodic
// image; a cell of a boundary plane is its own slot (fluid index or private slot); any other
// solid cell is a link slot.  map[c] (every cell of the halo-1 box) is the slot a boundary
// condition addresses: >= 0 a slot the cell owns, <= -2 the image's slot -map-2 (a periodic
// ghost), -1 none.  The update is the dense layout's slot for slot, so every fluid and
// boundary-plane value is bit-identical to it.
//
// The porous plate rewrites interior slots of its planes after the halo exchange, so the
// exchanged ghost copies of those slots keep the values from before the plate (the
// reference exchanges, then applies the plate).  A ghost that aliased its image would see
// the plate's value instead; the y ghosts of the `ghost_planes` therefore own private slots
// and `wrap` lists, per (i, k) of those planes, the slots {ghost j = 0, image j = ny,
// ghost j = ny + 1, image j = 1} that the device exchanges like the dense y-face exchange
// (the five directions that cross the face; pull after an even step, push after an odd one).
struct MpListLayout : ListLayout {
    std::vector<int32_t> map;
    std::vector<int32_t> wrap;   // [nwrap][4]
    int64_t nplane = 0;
    int64_t spare = 0;
    int64_t nwrap = 0;
};

bool build_mp_list_layout(const int8_t *walls_h2, int nx, int ny, int nz, int jper, int kper,
                          const std::vector<int> &planes, const std::vector<int> &ghost_planes, MpListLayout &out,
                          std::string &why);

}  // namespace mflbm
