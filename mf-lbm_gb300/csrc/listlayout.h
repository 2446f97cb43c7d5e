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

}  // namespace mflbm
