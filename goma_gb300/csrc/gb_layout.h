// Host-side layout of one Q2/P1 problem: DOF map, CSR sparsity, the
// node-neighbour offsets the assembly kernels use to find CSR slots, the
// Dirichlet marks and the element colouring.  Built once per problem.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gb_problem.h"

namespace gb {

struct Layout {
  int dim = 0, nn = 0, centroid = 0, nvn = 0, npres = 0, nloc = 0, energy = 0;
  int nspec = 0;  // species; nodal fields are u..(w), T, Y_0..Y_{nspec-1}
  int num_nodes = 0, num_elems = 0, N = 0;
  int64_t nnz = 0;              // CSR entries, diagonal included
  std::vector<int> fu;          // first unknown per node (num_nodes + 1)
  std::vector<int64_t> rowptr;  // N + 1
  std::vector<int> colidx;      // nnz, ascending per row
  // Node graph: neighbours of node n are nbr_node[nbr_ptr[n] .. nbr_ptr[n+1]),
  // ascending.  nbr_off / nbr_offT give the offset, within any row of node n,
  // of neighbour s's first unknown (nbr_offT for the energy row, which skips
  // pressure columns).
  std::vector<int> nbr_ptr, nbr_node, nbr_off, nbr_offT;
  // For element e and local nodes k, l: index s of node conn[e][l] in the
  // neighbour list of node conn[e][k].
  std::vector<uint16_t> elem_nslot;
  std::vector<uint8_t> dbc;     // 1 on Dirichlet / pressure-datum unknowns
  std::vector<double> dbc_val;  // their values (later cards win)
  std::vector<int> color_ptr, color_elems;
};

// Returns 0 on success, -1 with a message in err.
int build_layout(const gb_problem_desc *d, Layout &L, std::string &err);
// The same matrix with node n renumbered perm[n] (unknowns stay grouped by
// node, in the same order within a node).  Fills the DOF map, CSR pattern
// and node graph of Lp (no mesh data: elem_nslot, Dirichlet marks and
// colours stay empty), umap (new unknown -> old unknown) and vmap (new CSR
// entry -> old CSR entry).
void permute_layout(const Layout &L, const std::vector<int> &perm, Layout &Lp,
                    std::vector<int> &umap, std::vector<int64_t> &vmap);
// A node order with few ILU(0) dependency levels: the nodes without
// pressure unknowns by greedy colours of the node graph, then the element
// centroid nodes (which carry the P1 pressures) by greedy colours of theirs,
// so that every pressure pivot comes after all velocities of its element.
// Returns perm (old node -> new node) and the number of colours.
int multicolour_order(const Layout &L, std::vector<int> &perm);
// Order in which a sync-free triangular sweep adds each row's off-node
// entries: the lower neighbours of node n (m < n) by ascending dependency
// level lev[m], the upper ones by ascending levu[m] (ties by node number),
// so the values a row needs first are the ones published longest ago.
// rel[p], for CSR position p of a row's off-node lower segment [rowptr[i],
// diag(i) - r) or upper segment [diag(i) + 1 + na, rowptr[i+1]), is the
// position within the same segment of the entry to take p-th.  Returns -1
// when a segment is longer than 65,535 entries.
int build_sweep_order(const Layout &L, const std::vector<int> &lev, const std::vector<int> &levu,
                      std::vector<uint16_t> &rel);
// MSR pattern of the reference (diagonal first, off-diagonals ascending).
void layout_msr_pattern(const Layout &L, int *ija);
int64_t layout_msr_length(const Layout &L);

}  // namespace gb
