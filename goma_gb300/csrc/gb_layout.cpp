// DOF map, sparsity and colouring of a Q2/P1 mesh.
//
// Unknown numbering restates Index_Solution (src/mm_unknown_map.c:5268):
// node by node; per node the velocity components, then T when the energy
// equation is on, then the species Y_0.., and at an element's centroid node
// its dim+1 P1 pressure unknowns (variable types ascending,
// include/rf_fem_const.h:174-200).  The coupling graph restates build_node_node
// (src/exo_conn.c:204) and find_MSR_problem_graph (src/mm_fill_util.c:3229):
// an unknown couples with every unknown of every node that shares an
// element with its node; a centroid node also couples with the centroid
// nodes of its element's face neighbours (src/exo_conn.c:300-330); the
// energy equation does not couple with pressure (set_interaction_masks,
// src/mm_unknown_map.c:1125).  Rows keep the diagonal in place (CSR); the
// reference's MSR form is the same order with the diagonal pulled out.
#include "gb_layout.h"

#include <algorithm>
#include <cstring>

namespace gb {

int build_layout(const gb_problem_desc *d, Layout &L, std::string &err) {
  if (!d || (d->dim != 2 && d->dim != 3)) {
    err = "dim must be 2 (QUAD9) or 3 (HEX27)";
    return -1;
  }
  if (d->num_nodes <= 0 || d->num_elems <= 0 || !d->coords || !d->conn) {
    err = "empty mesh";
    return -1;
  }
  L.dim = d->dim;
  L.nn = d->dim == 2 ? 9 : 27;
  L.centroid = d->dim == 2 ? 8 : 20;
  L.energy = d->energy ? 1 : 0;
  if (d->num_species < 0 || d->num_species > GB_MAX_SPECIES) {
    err = "num_species must be in [0, GB_MAX_SPECIES]";
    return -1;
  }
  L.nspec = d->num_species;
  for (int w = 0; w < L.nspec; w++) {
    const int m = d->mat.species_source_model[w];
    if (m != GB_SPECIES_SOURCE_NONE && m != GB_SPECIES_SOURCE_CONSTANT &&
        m != GB_SPECIES_SOURCE_ARRHENIUS) {
      err = "unknown species source model";
      return -1;
    }
    if (m == GB_SPECIES_SOURCE_ARRHENIUS) {
      const double s = d->mat.species_source[w][3];
      if (!L.energy || !(s >= 0.0 && s < L.nspec && s == (int)s)) {
        err = "an Arrhenius species source needs the energy equation and a valid species index";
        return -1;
      }
    }
  }
  L.nvn = d->dim + L.energy + L.nspec;
  L.npres = d->dim + 1;
  L.nloc = L.nvn * L.nn + L.npres;
  L.num_nodes = d->num_nodes;
  L.num_elems = d->num_elems;
  const int nn = L.nn, nnod = L.num_nodes, ne = L.num_elems;
  for (int64_t i = 0; i < (int64_t)ne * nn; i++) {
    if (d->conn[i] < 0 || d->conn[i] >= nnod) {
      err = "connectivity references a node outside [0, num_nodes)";
      return -1;
    }
  }
  // centroid nodes
  std::vector<int> cent_elem(nnod, -1);
  for (int e = 0; e < ne; e++) {
    int c = d->conn[(int64_t)e * nn + L.centroid];
    if (cent_elem[c] != -1) {
      err = "a centroid node is shared by two elements";
      return -1;
    }
    cent_elem[c] = e;
  }
  L.fu.assign(nnod + 1, 0);
  for (int n = 0; n < nnod; n++) L.fu[n + 1] = L.fu[n] + L.nvn + (cent_elem[n] >= 0 ? L.npres : 0);
  if ((int64_t)L.fu[nnod] > 2000000000LL) {
    err = "more than 2e9 unknowns";
    return -1;
  }
  L.N = L.fu[nnod];
  // node -> elements
  std::vector<int> ne_ptr(nnod + 1, 0);
  for (int64_t i = 0; i < (int64_t)ne * nn; i++) ne_ptr[d->conn[i] + 1]++;
  for (int n = 0; n < nnod; n++) ne_ptr[n + 1] += ne_ptr[n];
  std::vector<int> ne_list(ne_ptr[nnod]);
  {
    std::vector<int> fill(nnod, 0);
    for (int e = 0; e < ne; e++)
      for (int k = 0; k < nn; k++) {
        int n = d->conn[(int64_t)e * nn + k];
        ne_list[ne_ptr[n] + fill[n]++] = e;
      }
  }
  const int side0 = d->dim == 2 ? 4 : 21, side1 = d->dim == 2 ? 8 : 27;
  // node graph
  L.nbr_ptr.assign(nnod + 1, 0);
  std::vector<std::vector<int>> nbrs(nnod);
  std::vector<int> tmp;
  for (int n = 0; n < nnod; n++) {
    tmp.clear();
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; q++) {
      const int *c = d->conn + (int64_t)ne_list[q] * nn;
      tmp.insert(tmp.end(), c, c + nn);
    }
    if (cent_elem[n] >= 0 && ne_ptr[n + 1] - ne_ptr[n] == 1) {
      int e = cent_elem[n];
      for (int k = side0; k < side1; k++) {
        int m = d->conn[(int64_t)e * nn + k];
        for (int q = ne_ptr[m]; q < ne_ptr[m + 1]; q++) {
          int f = ne_list[q];
          if (f != e) tmp.push_back(d->conn[(int64_t)f * nn + L.centroid]);
        }
      }
    }
    std::sort(tmp.begin(), tmp.end());
    tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
    if (tmp.size() > 65535) {
      err = "node with more than 65535 neighbours";
      return -1;
    }
    nbrs[n] = tmp;
    L.nbr_ptr[n + 1] = L.nbr_ptr[n] + (int)tmp.size();
  }
  L.nbr_node.resize(L.nbr_ptr[nnod]);
  L.nbr_off.resize(L.nbr_ptr[nnod]);
  L.nbr_offT.resize(L.nbr_ptr[nnod]);
  std::vector<int64_t> len_all(nnod), len_T(nnod);
  for (int n = 0; n < nnod; n++) {
    int off = 0, offT = 0;
    for (size_t s = 0; s < nbrs[n].size(); s++) {
      int m = nbrs[n][s], q = L.nbr_ptr[n] + (int)s;
      L.nbr_node[q] = m;
      L.nbr_off[q] = off;
      L.nbr_offT[q] = offT;
      off += L.fu[m + 1] - L.fu[m];
      offT += L.nvn;
    }
    len_all[n] = off;
    len_T[n] = offT;
  }
  // CSR
  L.rowptr.assign((size_t)L.N + 1, 0);
  for (int n = 0; n < nnod; n++)
    for (int i = L.fu[n]; i < L.fu[n + 1]; i++) {
      bool rowT = L.energy && (i - L.fu[n]) == L.dim;
      L.rowptr[i + 1] = rowT ? len_T[n] : len_all[n];
    }
  for (int i = 0; i < L.N; i++) L.rowptr[i + 1] += L.rowptr[i];
  L.nnz = L.rowptr[L.N];
  L.colidx.resize((size_t)L.nnz);
  for (int n = 0; n < nnod; n++)
    for (int i = L.fu[n]; i < L.fu[n + 1]; i++) {
      bool rowT = L.energy && (i - L.fu[n]) == L.dim;
      int64_t pos = L.rowptr[i];
      for (int m : nbrs[n])
        for (int j = L.fu[m]; j < L.fu[m + 1]; j++) {
          if (rowT && j - L.fu[m] >= L.nvn) continue;
          L.colidx[pos++] = j;
        }
    }
  // element -> neighbour slots
  L.elem_nslot.resize((size_t)ne * nn * nn);
  for (int e = 0; e < ne; e++) {
    const int *c = d->conn + (int64_t)e * nn;
    for (int k = 0; k < nn; k++) {
      const std::vector<int> &nb = nbrs[c[k]];
      for (int l = 0; l < nn; l++) {
        auto it = std::lower_bound(nb.begin(), nb.end(), c[l]);
        L.elem_nslot[((size_t)e * nn + k) * nn + l] = (uint16_t)(it - nb.begin());
      }
    }
  }
  // Dirichlet cards in order, later cards win (src/mm_bc.c:132)
  L.dbc.assign(L.N, 0);
  L.dbc_val.assign(L.N, 0.0);
  for (int c = 0; c < d->num_bc; c++) {
    int var = d->bc_var[c], off;
    if (var >= GB_VAR_U1 && var < GB_VAR_U1 + d->dim)
      off = var;
    else if (var == GB_VAR_T && L.energy)
      off = d->dim;
    else if (var == GB_VAR_T)
      continue;
    else if (var >= GB_VAR_Y(0) && var < GB_VAR_Y(0) + GB_MAX_SPECIES) {
      if (var - GB_VAR_Y(0) >= L.nspec) continue;
      off = d->dim + L.energy + (var - GB_VAR_Y(0));
    } else if (var == GB_VAR_P) {
      off = L.nvn;  // first pressure unknown of a centroid node
    } else {
      err = "Dirichlet card on an unsupported variable";
      return -1;
    }
    for (int q = d->bc_ptr[c]; q < d->bc_ptr[c + 1]; q++) {
      int n = d->bc_nodes[q];
      if (n < 0 || n >= nnod) {
        err = "Dirichlet node outside the mesh";
        return -1;
      }
      if (var == GB_VAR_P && L.fu[n + 1] - L.fu[n] <= L.nvn) {
        err = "pressure card on a node without pressure unknowns (not an element centroid)";
        return -1;
      }
      L.dbc[L.fu[n] + off] = 1;
      L.dbc_val[L.fu[n] + off] = d->bc_value[c];
    }
  }
  // PRESSURE DATUM: first pressure unknown of the element (src/mm_bc.c:418)
  if (d->pressure_datum_elem >= 0) {
    if (d->pressure_datum_elem >= ne) {
      err = "pressure datum element out of range";
      return -1;
    }
    int c = d->conn[(int64_t)d->pressure_datum_elem * nn + L.centroid];
    L.dbc[L.fu[c] + L.nvn] = 1;
    L.dbc_val[L.fu[c] + L.nvn] = d->pressure_datum_value;
  }
  // greedy colouring: elements sharing a node get different colours, so a
  // colour's elements write disjoint CSR rows
  std::vector<int> color(ne, -1);
  int ncol = 0;
  for (int e = 0; e < ne; e++) {
    uint64_t used = 0;
    const int *c = d->conn + (int64_t)e * nn;
    for (int k = 0; k < nn; k++)
      for (int q = ne_ptr[c[k]]; q < ne_ptr[c[k] + 1]; q++) {
        int f = ne_list[q];
        if (color[f] >= 0 && color[f] < 64) used |= 1ull << color[f];
      }
    int col = 0;
    while (col < 64 && (used >> col & 1ull)) col++;
    if (col >= 64) {
      err = "element colouring needs more than 64 colours";
      return -1;
    }
    color[e] = col;
    ncol = std::max(ncol, col + 1);
  }
  L.color_ptr.assign(ncol + 1, 0);
  for (int e = 0; e < ne; e++) L.color_ptr[color[e] + 1]++;
  for (int k = 0; k < ncol; k++) L.color_ptr[k + 1] += L.color_ptr[k];
  L.color_elems.resize(ne);
  {
    std::vector<int> fill(ncol, 0);
    for (int e = 0; e < ne; e++) L.color_elems[L.color_ptr[color[e]] + fill[color[e]]++] = e;
  }
  return 0;
}

int64_t layout_msr_length(const Layout &L) { return (int64_t)L.N + 1 + (L.nnz - L.N); }

void layout_msr_pattern(const Layout &L, int *ija) {
  int64_t pos = (int64_t)L.N + 1;
  for (int i = 0; i < L.N; i++) {
    ija[i] = (int)pos;
    for (int64_t k = L.rowptr[i]; k < L.rowptr[i + 1]; k++)
      if (L.colidx[k] != i) ija[pos++] = L.colidx[k];
  }
  ija[L.N] = (int)pos;
}

}  // namespace gb

namespace gb {

int multicolour_order(const Layout &L, std::vector<int> &perm) {
  const int nn = L.num_nodes;
  std::vector<char> cent(nn);
  for (int n = 0; n < nn; n++) cent[n] = (L.fu[n + 1] - L.fu[n]) > L.nvn;
  std::vector<int> colour(nn, -1);
  int ncol[2] = {0, 0};
  std::vector<char> used;
  for (int pass = 0; pass < 2; pass++) {
    for (int n = 0; n < nn; n++) {
      if (cent[n] != pass) continue;
      used.assign(ncol[pass] + 1, 0);
      for (int q = L.nbr_ptr[n]; q < L.nbr_ptr[n + 1]; q++) {
        const int m = L.nbr_node[q];
        if (cent[m] == pass && colour[m] >= 0) used[colour[m]] = 1;
      }
      int c = 0;
      while (used[c]) c++;
      colour[n] = c;
      if (c + 1 > ncol[pass]) ncol[pass] = c + 1;
    }
  }
  // order: non-centroid colours, then centroid colours; ascending node id within
  std::vector<int> count(ncol[0] + ncol[1] + 1, 0);
  auto key = [&](int n) { return cent[n] ? ncol[0] + colour[n] : colour[n]; };
  for (int n = 0; n < nn; n++) count[key(n) + 1]++;
  for (size_t k = 1; k < count.size(); k++) count[k] += count[k - 1];
  perm.assign(nn, 0);
  for (int n = 0; n < nn; n++) perm[n] = count[key(n)]++;
  return ncol[0] + ncol[1];
}

void permute_layout(const Layout &L, const std::vector<int> &perm, Layout &Lp,
                    std::vector<int> &umap, std::vector<int64_t> &vmap) {
  const int nn = L.num_nodes;
  std::vector<int> iperm(nn);
  for (int n = 0; n < nn; n++) iperm[perm[n]] = n;
  Lp.dim = L.dim;
  Lp.nn = L.nn;
  Lp.centroid = L.centroid;
  Lp.nvn = L.nvn;
  Lp.npres = L.npres;
  Lp.nloc = L.nloc;
  Lp.energy = L.energy;
  Lp.nspec = L.nspec;
  Lp.num_nodes = nn;
  Lp.num_elems = L.num_elems;
  Lp.N = L.N;
  Lp.fu.assign(nn + 1, 0);
  for (int np = 0; np < nn; np++) {
    const int n = iperm[np];
    Lp.fu[np + 1] = Lp.fu[np] + (L.fu[n + 1] - L.fu[n]);
  }
  umap.assign(L.N, 0);
  for (int np = 0; np < nn; np++)
    for (int d = 0; d < Lp.fu[np + 1] - Lp.fu[np]; d++) umap[Lp.fu[np] + d] = L.fu[iperm[np]] + d;
  // node graph in the new numbering
  Lp.nbr_ptr.assign(nn + 1, 0);
  for (int np = 0; np < nn; np++) {
    const int n = iperm[np];
    Lp.nbr_ptr[np + 1] = Lp.nbr_ptr[np] + (L.nbr_ptr[n + 1] - L.nbr_ptr[n]);
  }
  const size_t ne = (size_t)Lp.nbr_ptr[nn];
  Lp.nbr_node.resize(ne);
  Lp.nbr_off.resize(ne);
  Lp.nbr_offT.resize(ne);
  std::vector<int> oldslot(ne);  // new slot -> old slot index (absolute)
#pragma omp parallel for schedule(dynamic, 256)
  for (int np = 0; np < nn; np++) {
    const int n = iperm[np];
    const int b0 = L.nbr_ptr[n], cnt = L.nbr_ptr[n + 1] - b0, q0 = Lp.nbr_ptr[np];
    std::vector<std::pair<int, int>> v(cnt);
    for (int s = 0; s < cnt; s++) v[s] = {perm[L.nbr_node[b0 + s]], b0 + s};
    std::sort(v.begin(), v.end());
    int off = 0, offT = 0;
    for (int s = 0; s < cnt; s++) {
      const int mp = v[s].first, m = iperm[mp];
      Lp.nbr_node[q0 + s] = mp;
      Lp.nbr_off[q0 + s] = off;
      Lp.nbr_offT[q0 + s] = offT;
      oldslot[q0 + s] = v[s].second;
      off += L.fu[m + 1] - L.fu[m];
      offT += L.nvn;
    }
  }
  // CSR: row lengths are those of the old rows
  Lp.rowptr.assign((size_t)L.N + 1, 0);
  for (int i = 0; i < L.N; i++) Lp.rowptr[i + 1] = L.rowptr[umap[i] + 1] - L.rowptr[umap[i]];
  for (int i = 0; i < L.N; i++) Lp.rowptr[i + 1] += Lp.rowptr[i];
  Lp.nnz = Lp.rowptr[L.N];
  Lp.colidx.resize((size_t)Lp.nnz);
  vmap.resize((size_t)Lp.nnz);
#pragma omp parallel for schedule(dynamic, 256)
  for (int np = 0; np < nn; np++) {
    const int n = iperm[np];
    for (int d = 0; d < Lp.fu[np + 1] - Lp.fu[np]; d++) {
      const int ip = Lp.fu[np] + d, i = L.fu[n] + d;
      const bool rowT = L.energy && d == L.dim;
      int64_t pos = Lp.rowptr[ip];
      for (int q = Lp.nbr_ptr[np]; q < Lp.nbr_ptr[np + 1]; q++) {
        const int mp = Lp.nbr_node[q], m = iperm[mp], oq = oldslot[q];
        const int nd = rowT ? L.nvn : L.fu[m + 1] - L.fu[m];
        const int64_t ob = L.rowptr[i] + (rowT ? L.nbr_offT[oq] : L.nbr_off[oq]);
        for (int e = 0; e < nd; e++) {
          Lp.colidx[(size_t)pos] = Lp.fu[mp] + e;
          vmap[(size_t)pos] = ob + e;
          pos++;
        }
      }
    }
  }
}

}  // namespace gb

namespace gb {

int build_sweep_order(const Layout &L, const std::vector<int> &lev, const std::vector<int> &levu,
                      std::vector<uint16_t> &rel) {
  rel.assign((size_t)L.nnz, 0);
  const int Tr = L.energy ? L.dim : -1;
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(| : bad)
  for (int n = 0; n < L.num_nodes; n++) {
    const int b = L.nbr_ptr[n], e = L.nbr_ptr[n + 1];
    // neighbour slots below and above n, by level then node number
    std::vector<int> lo, up;
    for (int s = b; s < e; s++) {
      const int m = L.nbr_node[s];
      if (m < n) lo.push_back(s);
      if (m > n) up.push_back(s);
    }
    std::stable_sort(lo.begin(), lo.end(), [&](int a, int c) {
      return lev[L.nbr_node[a]] < lev[L.nbr_node[c]];
    });
    std::stable_sort(up.begin(), up.end(), [&](int a, int c) {
      return levu[L.nbr_node[a]] < levu[L.nbr_node[c]];
    });
    const int f0 = L.fu[n], nr = L.fu[n + 1] - f0;
    for (int r = 0; r < nr; r++) {
      const int64_t i = f0 + r;
      const bool rowT = r == Tr;
      auto off = [&](int s) { return rowT ? L.nbr_offT[s] : L.nbr_off[s]; };
      auto len = [&](int s) {
        const int q = L.nbr_node[s];
        return rowT ? L.nvn : L.fu[q + 1] - L.fu[q];
      };
      // lower segment starts at the row start; upper at the first column
      // after the own node's block
      int self = b;
      while (L.nbr_node[self] != n) self++;
      const int64_t lo0 = L.rowptr[i];
      const int64_t up0 = L.rowptr[i] + off(self) + len(self);
      int64_t k = 0;
      for (int s : lo)
        for (int t = 0; t < len(s); t++) {
          const int64_t v = off(s) + t;
          if (v > 65535) bad = 1;
          rel[(size_t)(lo0 + k++)] = (uint16_t)v;
        }
      k = 0;
      const int64_t base = off(self) + len(self);
      for (int s : up)
        for (int t = 0; t < len(s); t++) {
          const int64_t v = off(s) + t - base;
          if (v > 65535) bad = 1;
          rel[(size_t)(up0 + k++)] = (uint16_t)v;
        }
    }
  }
  return bad ? -1 : 0;
}

}  // namespace gb
