// Problem context: device copies of the layout, the reference-element
// tables, the assembly driver and the C ABI of include/gb_newton.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gb_newton.h"
#include "gb_context.h"

namespace gb {

thread_local std::string g_err;

int fail(const std::string &m) {
  g_err = m;
  return -1;
}
int cuda_fail(cudaError_t e, const char *where) {
  g_err = std::string(where) + ": " + cudaGetErrorString(e);
  return -1;
}

// Reference-element tables at the Gauss points, in the reference's point
// order (src/el_elm_info.c:1748 QUAD9, :1802 HEX27) and with its literal
// constants (:1642 abscissa, :3484-3485 weights); Q2 basis as tensor
// products of the 1-D quadratic Lagrange polynomials on -1, 0, +1 (the
// polynomials of src/rf_shape.c:361 BIQUAD_QUAD and :1105 TRIQUAD_HEX).
static const int kLoc9[9][2] = {{0, 0}, {2, 0}, {2, 2}, {0, 2}, {1, 0},
                                {2, 1}, {1, 2}, {0, 1}, {1, 1}};
static const int kLoc27[27][3] = {
    {0, 0, 0}, {2, 0, 0}, {2, 2, 0}, {0, 2, 0}, {0, 0, 2}, {2, 0, 2}, {2, 2, 2},
    {0, 2, 2}, {1, 0, 0}, {2, 1, 0}, {1, 2, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 1},
    {2, 2, 1}, {0, 2, 1}, {1, 0, 2}, {2, 1, 2}, {1, 2, 2}, {0, 1, 2}, {1, 1, 1},
    {1, 1, 0}, {1, 1, 2}, {0, 1, 1}, {2, 1, 1}, {1, 0, 1}, {1, 2, 1}};
static const double kPt[3] = {0.77459666924148340428, 0.0, -0.77459666924148340428};
static const double kWt[3] = {0.55555555555555555556, 0.88888888888888888888,
                              0.55555555555555555556};
static double lag(int g, double s) {
  return g == 0 ? 0.5 * s * (s - 1.0) : (g == 1 ? 1.0 - s * s : 0.5 * s * (s + 1.0));
}
static double dlag(int g, double s) { return g == 0 ? s - 0.5 : (g == 1 ? -2.0 * s : s + 0.5); }

void build_tables(int dim, std::vector<double> &phi, std::vector<double> &dphi,
                  std::vector<double> &w) {
  const int nn = dim == 2 ? 9 : 27, nq = nn;
  phi.assign(nq * nn, 0.0);
  dphi.assign(nq * nn * dim, 0.0);
  w.assign(nq, 0.0);
  for (int q = 0; q < nq; q++) {
    const int is = q % 3, it = (q % 9) / 3, iu = q / 9;
    const double s = kPt[is], t = kPt[it], u = dim == 3 ? kPt[iu] : 0.0;
    w[q] = dim == 3 ? kWt[is] * kWt[it] * kWt[iu] : kWt[is] * kWt[it];
    for (int k = 0; k < nn; k++) {
      if (dim == 2) {
        const int gx = kLoc9[k][0], gy = kLoc9[k][1];
        phi[q * nn + k] = lag(gx, s) * lag(gy, t);
        dphi[(q * nn + k) * 2 + 0] = dlag(gx, s) * lag(gy, t);
        dphi[(q * nn + k) * 2 + 1] = lag(gx, s) * dlag(gy, t);
      } else {
        const int gx = kLoc27[k][0], gy = kLoc27[k][1], gz = kLoc27[k][2];
        phi[q * nn + k] = lag(gx, s) * lag(gy, t) * lag(gz, u);
        dphi[(q * nn + k) * 3 + 0] = dlag(gx, s) * lag(gy, t) * lag(gz, u);
        dphi[(q * nn + k) * 3 + 1] = lag(gx, s) * dlag(gy, t) * lag(gz, u);
        dphi[(q * nn + k) * 3 + 2] = lag(gx, s) * lag(gy, t) * dlag(gz, u);
      }
    }
  }
}

template <class T>
static int upload(T **dst, const std::vector<T> &src, const char *what) {
  size_t n = src.size() ? src.size() : 1;
  cudaError_t e = cudaMalloc((void **)dst, n * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(e, what);
  if (src.size()) {
    e = cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, what);
  }
  return 0;
}

// CSR value k of row i lands at MSR position i (diagonal) or
// N + 1 + k - i - (k > diag(i)).
__global__ void csr_to_msr_kernel(int N, const int64_t *__restrict__ rowptr,
                                  const int *__restrict__ colidx, const double *__restrict__ vals,
                                  double *__restrict__ msr) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= N) return;
  const int i = warp;
  const int64_t r0 = rowptr[i], r1 = rowptr[i + 1];
  for (int64_t k = r0 + lane; k < r1; k += 32) {
    const int c = colidx[k];
    if (c == i) {
      msr[i] = vals[k];
    } else {
      const int64_t pos = (int64_t)N + 1 + k - i - (c > i ? 1 : 0);
      msr[pos] = vals[k];
    }
  }
  if (i == 0 && lane == 0) msr[N] = 0.0;
}

// dst[0 .. n) = src[0 .. n), both 16-byte aligned: 16-byte stores
__global__ void copy16_kernel(const double *__restrict__ src, double *__restrict__ dst,
                              int64_t n) {
  const int64_t n2 = n >> 1;
  const double2 *s2 = reinterpret_cast<const double2 *>(src);
  double2 *d2 = reinterpret_cast<double2 *>(dst);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2;
       i += (int64_t)gridDim.x * blockDim.x)
    d2[i] = s2[i];
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) dst[n - 1] = src[n - 1];
}

Context::~Context() {
  void *ptrs[] = {d_coords, d_conn,   d_fu,     d_dbc,     d_dbc_val, d_rowptr, d_colidx,
                  d_nbr_ptr, d_nbr_off, d_nbr_offT, d_nbr_node, d_nslot, d_tab_phi, d_tab_dphi, d_tab_w,
                  d_tab_pt, d_tab_iso, d_color_elems, d_x, d_R, d_vals, d_status, d_msr,
                  d_elem_rho, d_side_elem, d_side_side, d_side_type, d_side_val};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (d_sf) cudaFree(d_sf);
  if (ev_k0) cudaEventDestroy(ev_k0);
  if (ev_k1) cudaEventDestroy(ev_k1);
  if (stream) cudaStreamDestroy(stream);
}

int Context::set_material(const gb_material &m) {
  if (m.viscosity_model != GB_VISC_NEWTONIAN && m.viscosity_model != GB_VISC_CARREAU)
    return fail("unsupported viscosity model");
  if (m.momentum_source_model != GB_SOURCE_CONSTANT &&
      m.momentum_source_model != GB_SOURCE_BOUSSINESQ)
    return fail("unsupported momentum source model");
  mat.density = m.density;
  mat.viscosity = m.viscosity;
  mat.mu0 = m.mu0;
  mat.mu_inf = m.mu_inf;
  mat.lambda = m.lambda;
  mat.aexp = m.aexp;
  mat.nexp = m.nexp;
  mat.heat_capacity = m.heat_capacity;
  mat.conductivity = m.conductivity;
  mat.source_model = m.momentum_source_model;
  for (int a = 0; a < 3; a++) mat.source[a] = m.momentum_source[a];
  mat.beta = m.volume_expansion;
  mat.Tref = m.reference_temperature;
  mat.nspec = L.nspec;
  for (int w = 0; w < GB_MAX_SPECIES; w++) {
    const bool on = w < L.nspec;
    const int model = on ? m.species_source_model[w] : GB_SPECIES_SOURCE_NONE;
    if (model != GB_SPECIES_SOURCE_NONE && model != GB_SPECIES_SOURCE_CONSTANT &&
        model != GB_SPECIES_SOURCE_ARRHENIUS)
      return fail("unsupported species source model");
    if (model == GB_SPECIES_SOURCE_ARRHENIUS) {
      const double src = m.species_source[w][3];
      if (!L.energy || !(src >= 0.0 && src < L.nspec && src == (int)src))
        return fail("an Arrhenius species source needs the energy equation and a valid species index");
    }
    mat.diff[w] = on ? m.diffusivity[w] : 0.0;
    mat.ssm[w] = model;
    for (int k = 0; k < 4; k++) mat.ssp[w][k] = on ? m.species_source[w][k] : 0.0;
  }
  if (m.heat_source_model != GB_HEAT_SOURCE_NONE &&
      m.heat_source_model != GB_HEAT_SOURCE_CONSTANT &&
      m.heat_source_model != GB_HEAT_SOURCE_EXPONENTIAL)
    return fail("unsupported heat source model");
  mat.hsm = L.energy ? m.heat_source_model : GB_HEAT_SOURCE_NONE;
  mat.hs[0] = m.heat_source[0];
  mat.hs[1] = m.heat_source[1];
  carreau = m.viscosity_model == GB_VISC_CARREAU;
  desc.mat = m;
  return 0;
}

int Context::init(const gb_problem_desc *d) {
  desc = *d;
  if (build_layout(d, L, g_err) != 0) return -1;
  if (set_material(d->mat)) return -1;

  cudaError_t e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
  std::vector<double> coords(d->coords, d->coords + (size_t)d->num_nodes * d->dim);
  std::vector<int> conn(d->conn, d->conn + (size_t)d->num_elems * L.nn);
  std::vector<double> tphi, tdphi, tw;
  build_tables(L.dim, tphi, tdphi, tw);
  std::vector<double> tpt(kPt, kPt + 3);
  if (upload(&d_coords, coords, "coords") || upload(&d_conn, conn, "conn") ||
      upload(&d_fu, L.fu, "fu") || upload(&d_dbc, L.dbc, "dbc") ||
      upload(&d_dbc_val, L.dbc_val, "dbc_val") || upload(&d_rowptr, L.rowptr, "rowptr") ||
      upload(&d_colidx, L.colidx, "colidx") || upload(&d_nbr_ptr, L.nbr_ptr, "nbr_ptr") ||
      upload(&d_nbr_off, L.nbr_off, "nbr_off") || upload(&d_nbr_offT, L.nbr_offT, "nbr_offT") ||
      upload(&d_nbr_node, L.nbr_node, "nbr_node") ||
      upload(&d_nslot, L.elem_nslot, "elem_nslot") || upload(&d_tab_phi, tphi, "tab") ||
      upload(&d_tab_dphi, tdphi, "tab") || upload(&d_tab_w, tw, "tab") ||
      upload(&d_tab_pt, tpt, "tab") || upload(&d_color_elems, L.color_elems, "colors"))
    return -1;
  if (L.dim == 3) {
    std::vector<double> iso(112 * 28);
    build_iso_table(tphi.data(), tdphi.data(), iso.data());
    if (upload(&d_tab_iso, iso, "tab")) return -1;
    double ell[9], dell[9];
    for (int a = 0; a < 3; a++)
      for (int g = 0; g < 3; g++) {
        ell[a * 3 + g] = lag(a, kPt[g]);
        dell[a * 3 + g] = dlag(a, kPt[g]);
      }
    std::vector<SfTables> sft(1);
    build_sf_tables(tphi.data(), tdphi.data(), kLoc27, ell, dell, sft[0]);
    if (upload(&d_sf, sft, "tab")) return -1;
  }
  // integrated boundary conditions: the cards expanded to their sides
  if (d->num_ibc > 0) {
    std::vector<int> se, ss, st;
    std::vector<double> sv;
    const int maxside = L.dim == 2 ? 4 : 6;
    for (int c = 0; c < d->num_ibc; c++) {
      const int ty = d->ibc_type[c];
      if (ty != GB_IBC_QSIDE && ty != GB_IBC_QCONV && ty != GB_IBC_FLOW_PRESSURE)
        return fail("unsupported integrated boundary condition");
      if (ty != GB_IBC_FLOW_PRESSURE && !L.energy)
        return fail("a QSIDE or QCONV condition needs the energy equation");
      for (int k = d->ibc_ptr[c]; k < d->ibc_ptr[c + 1]; k++) {
        if (d->ibc_elem[k] < 0 || d->ibc_elem[k] >= L.num_elems || d->ibc_side[k] < 1 ||
            d->ibc_side[k] > maxside)
          return fail("integrated boundary condition side out of range");
        se.push_back(d->ibc_elem[k]);
        ss.push_back(d->ibc_side[k]);
        st.push_back(ty);
        sv.push_back(d->ibc_value[2 * c]);
        sv.push_back(d->ibc_value[2 * c + 1]);
      }
    }
    num_sides = (int)se.size();
    if (num_sides > 0 &&
        (upload(&d_side_elem, se, "sides") || upload(&d_side_side, ss, "sides") ||
         upload(&d_side_type, st, "sides") || upload(&d_side_val, sv, "sides")))
      return -1;
  }
  if ((e = cudaMalloc(&d_x, sizeof(double) * L.N)) != cudaSuccess) return cuda_fail(e, "x");
  if ((e = cudaMalloc(&d_R, sizeof(double) * L.N)) != cudaSuccess) return cuda_fail(e, "R");
  if ((e = cudaMalloc(&d_vals, sizeof(double) * L.nnz)) != cudaSuccess)
    return cuda_fail(e, "CSR values");
  if ((e = cudaMalloc(&d_status, sizeof(int) * 2)) != cudaSuccess) return cuda_fail(e, "status");
  return reset_status();
}

int Context::reset_status() {
  int h[2] = {0, 0x7fffffff};
  cudaError_t e = cudaMemcpyAsync(d_status, h, sizeof(h), cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  return e == cudaSuccess ? 0 : cuda_fail(e, "status reset");
}

AsmArgs Context::args(const double *x, double *R, double *vals) const {
  AsmArgs a;
  a.coords = d_coords;
  a.conn = d_conn;
  a.fu = d_fu;
  a.dbc = d_dbc;
  a.rowptr = d_rowptr;
  a.nbr_ptr = d_nbr_ptr;
  a.nbr_off = d_nbr_off;
  a.nbr_offT = d_nbr_offT;
  a.elem_nslot = d_nslot;
  a.tab_phi = d_tab_phi;
  a.tab_dphi = d_tab_dphi;
  a.tab_w = d_tab_w;
  a.tab_pt = d_tab_pt;
  a.x = x;
  a.R = R;
  a.vals = vals;
  a.status = d_status;
  a.elem_rho = d_elem_rho;
  a.pofs = L.nvn;
  a.xdot = d_xdot;
  a.mass_c = d_xdot ? mass_c : 0.0;
  a.mat = mat;
  return a;
}

int Context::assemble(const double *x, double *R, double *vals, cudaStream_t st) {
  if (!st) st = stream;
  cudaError_t e = cudaMemsetAsync(R, 0, sizeof(double) * L.N, st);
  if (e == cudaSuccess && vals) e = cudaMemsetAsync(vals, 0, sizeof(double) * L.nnz, st);
  if (e != cudaSuccess) return cuda_fail(e, "assembly zeroing");
  AsmArgs a = args(x, R, vals);
  const int ncol = (int)L.color_ptr.size() - 1;
  if (timing) cudaEventRecord(ev_k0, st);
  const int kp = kernel_path(vals != nullptr);
  if (kp >= 2 && tc_grid == 0) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    tc_grid = 2 * sms;
  }
  for (int c = 0; c < ncol; c++) {
    const int n = L.color_ptr[c + 1] - L.color_ptr[c];
    if (kp == 4)
      e = launch_assemble_sf(a, L.energy != 0, d_sf, d_color_elems + L.color_ptr[c], n, tc_grid,
                             st);
    else if (kp == 3)
      e = launch_assemble_gemm(a, L.energy != 0, d_tab_iso, d_color_elems + L.color_ptr[c], n,
                               tc_grid, st);
    else if (kp == 2)
      e = launch_assemble_tc(a, L.energy != 0, carreau, d_color_elems + L.color_ptr[c], n,
                             tc_grid, st);
    else
      e = launch_assemble(a, L.dim, L.energy != 0, carreau, vals != nullptr,
                          d_color_elems + L.color_ptr[c], n, st);
    if (e != cudaSuccess) return cuda_fail(e, "assembly launch");
    if (L.nspec > 0) {
      e = launch_assemble_species(a, L.dim, L.energy != 0, vals != nullptr,
                                  d_color_elems + L.color_ptr[c], n, st);
      if (e != cudaSuccess) return cuda_fail(e, "species assembly launch");
    }
  }
  if (num_sides > 0) {
    SideArgs sa{num_sides, d_side_elem, d_side_side, d_side_type, d_side_val};
    e = launch_assemble_sides(a, sa, L.dim, L.energy != 0, st);
    if (e != cudaSuccess) return cuda_fail(e, "boundary condition launch");
  }
  if (timing) {
    cudaEventRecord(ev_k1, st);
    cudaEventSynchronize(ev_k1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev_k0, ev_k1);
    kernel_ms += ms;
    kernel_launches += ncol * (L.nspec > 0 ? 2 : 1);
  }
  return 0;
}

int Context::kernel_path(bool jacobian) const {
  if (L.dim != 3) return 1;
  // a heat source: the scalar kernel
  if (mat.hsm != GB_HEAT_SOURCE_NONE) return 1;
  const bool gemm_ok = !carreau && mat.viscosity > 0.0;
  // per-element densities and transient terms: the scalar and the
  // sum-factorised kernels only
  if (d_elem_rho || d_xdot) return gemm_ok && path != 1 ? 4 : 1;
  if (path == 0) return gemm_ok ? 4 : 1;
  if (path == 3 || path == 4) return gemm_ok ? path : 1;
  return jacobian ? path : 1;
}

int Context::check_status() {
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_fail(e, "stream");
  int h[2];
  e = cudaMemcpy(h, d_status, sizeof(h), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "status");
  if (reset_status()) return -1;
  if (h[0] > 0) {
    char buf[160];
    snprintf(buf, sizeof buf, "%d element(s) with non-positive Jacobian determinant (first %d)",
             h[0], h[1]);
    return fail(buf);
  }
  return 0;
}

int Context::to_msr_host(const double *vals, double *a_msr) {
  cudaError_t e;
  const int64_t len = layout_msr_length(L);
  if (!d_msr) {
    e = cudaMalloc(&d_msr, sizeof(double) * len);
    if (e != cudaSuccess) return cuda_fail(e, "msr buffer");
  }
  const int threads = 256, blocks = (int)(((int64_t)L.N * 32 + threads - 1) / threads);
  csr_to_msr_kernel<<<blocks, threads, 0, stream>>>(L.N, d_rowptr, d_colidx, vals, d_msr);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "csr_to_msr");
  // A page-locked destination is written by a copy kernel with aligned
  // 16-byte stores over the host link: on GB300 that reached ~193 GB/s
  // into any page-locked buffer, where the copy engine's rate depended on
  // how the host memory was allocated (~90 GB/s into some) and the
  // conversion kernel's unaligned row stores reached ~151 GB/s.
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, a_msr) == cudaSuccess && at.type == cudaMemoryTypeHost &&
      at.devicePointer && ((uintptr_t)at.devicePointer & 15) == 0) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    copy16_kernel<<<4 * std::max(sms, 1), 256, 0, stream>>>(
        d_msr, static_cast<double *>(at.devicePointer), len);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "msr export");
  } else {
    cudaGetLastError();  // an unregistered (pageable) pointer is not an error here
    e = cudaMemcpyAsync(a_msr, d_msr, sizeof(double) * len, cudaMemcpyDeviceToHost, stream);
    if (e != cudaSuccess) return cuda_fail(e, "msr copy");
  }
  e = cudaStreamSynchronize(stream);
  return e == cudaSuccess ? 0 : cuda_fail(e, "msr export");
}

}  // namespace gb

using gb::Context;
using gb::fail;
using gb::cuda_fail;


extern "C" {

const char *gb_last_error(void) { return gb::g_err.c_str(); }

int gb_create(const gb_problem_desc *desc, gb_ctx **out) {
  if (!out) return fail("out is NULL");
  *out = nullptr;
  gb_ctx *h = new (std::nothrow) gb_ctx;
  if (!h) return fail("out of host memory");
  if (h->c.init(desc) != 0) {
    delete h;
    return -1;
  }
  *out = h;
  return 0;
}

void gb_destroy(gb_ctx *ctx) { delete ctx; }

int gb_num_unknowns(const gb_ctx *ctx) { return ctx ? ctx->c.L.N : -1; }
long long gb_msr_length(const gb_ctx *ctx) { return ctx ? gb::layout_msr_length(ctx->c.L) : -1; }
long long gb_csr_nnz(const gb_ctx *ctx) { return ctx ? ctx->c.L.nnz : -1; }
int gb_num_colors(const gb_ctx *ctx) { return ctx ? (int)ctx->c.L.color_ptr.size() - 1 : -1; }

int gb_msr_pattern(const gb_ctx *ctx, int *ija) {
  if (!ctx || !ija) return fail("NULL argument");
  if (gb::layout_msr_length(ctx->c.L) > 2147483647LL)
    return fail("MSR length exceeds the reference's 32-bit int indexing");
  gb::layout_msr_pattern(ctx->c.L, ija);
  return 0;
}

int gb_msr_pattern_host(const gb_problem_desc *desc, int *ija, long long *msr_length) {
  gb::Layout L;
  if (gb::build_layout(desc, L, gb::g_err) != 0) return -1;
  const long long len = gb::layout_msr_length(L);
  if (msr_length) *msr_length = len;
  if (len > 2147483647LL) return fail("MSR length exceeds the reference's 32-bit int indexing");
  if (ija) gb::layout_msr_pattern(L, ija);
  return 0;
}

int gb_ilu_permutation_host(const gb_problem_desc *desc, int *perm, int *num_colours, int *umap,
                            long long *rowptr, int *colidx, long long *vmap) {
  gb::Layout L, Lp;
  if (gb::build_layout(desc, L, gb::g_err) != 0) return -1;
  std::vector<int> pm, um;
  std::vector<int64_t> vm;
  const int nc = gb::multicolour_order(L, pm);
  if (num_colours) *num_colours = nc;
  if (perm) memcpy(perm, pm.data(), sizeof(int) * pm.size());
  if (!umap && !rowptr && !colidx && !vmap) return 0;
  gb::permute_layout(L, pm, Lp, um, vm);
  if (umap) memcpy(umap, um.data(), sizeof(int) * um.size());
  if (rowptr)
    for (int i = 0; i <= Lp.N; i++) rowptr[i] = Lp.rowptr[i];
  if (colidx) memcpy(colidx, Lp.colidx.data(), sizeof(int) * Lp.colidx.size());
  if (vmap)
    for (size_t k = 0; k < vm.size(); k++) vmap[k] = vm[k];
  return 0;
}

int gb_sweep_order_host(const gb_problem_desc *desc, int ordering, unsigned short *rel,
                        int *lev, int *levu) {
  if (!desc || !rel) return fail("NULL argument");
  gb::Layout L, Lp;
  if (gb::build_layout(desc, L, gb::g_err) != 0) return -1;
  const gb::Layout *LP = &L;
  if (ordering == GB_ILU_MULTICOLOUR) {
    std::vector<int> pm, um;
    std::vector<int64_t> vm;
    gb::multicolour_order(L, pm);
    gb::permute_layout(L, pm, Lp, um, vm);
    LP = &Lp;
  }
  gb::IluSchedule S;
  gb::build_ilu_schedule(*LP, S);
  std::vector<uint16_t> r;
  if (gb::build_sweep_order(*LP, S.lev, S.levu, r)) return fail("a matrix row is too long");
  memcpy(rel, r.data(), sizeof(uint16_t) * r.size());
  if (lev) memcpy(lev, S.lev.data(), sizeof(int) * S.lev.size());
  if (levu) memcpy(levu, S.levu.data(), sizeof(int) * S.levu.size());
  return 0;
}

int gb_csr_pattern(const gb_ctx *ctx, long long *rowptr, int *colidx) {
  if (!ctx || !rowptr || !colidx) return fail("NULL argument");
  const gb::Layout &L = ctx->c.L;
  for (int i = 0; i <= L.N; i++) rowptr[i] = L.rowptr[i];
  memcpy(colidx, L.colidx.data(), sizeof(int) * L.colidx.size());
  return 0;
}

long long gb_csr_row(gb_ctx *ctx, const double *d_vals, int row, long long *start, int *cols,
                     double *vals, long long capacity) {
  if (!ctx) return fail("NULL argument");
  const gb::Layout &L = ctx->c.L;
  if (row < 0 || row >= L.N) return fail("row out of range");
  const int64_t b = L.rowptr[row], len = L.rowptr[row + 1] - b;
  if (start) *start = b;
  if (!cols && !vals) return len;
  if (len > capacity) return fail("row longer than the capacity given");
  if (cols) memcpy(cols, L.colidx.data() + b, sizeof(int) * (size_t)len);
  if (vals) {
    if (!d_vals) return fail("NULL device values");
    cudaError_t e = cudaMemcpyAsync(vals, d_vals + b, sizeof(double) * (size_t)len,
                                    cudaMemcpyDeviceToHost, ctx->c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->c.stream);
    if (e != cudaSuccess) return cuda_fail(e, "row copy");
  }
  return len;
}

int gb_first_unknown(const gb_ctx *ctx, int *fu) {
  if (!ctx || !fu) return fail("NULL argument");
  memcpy(fu, ctx->c.L.fu.data(), sizeof(int) * ctx->c.L.fu.size());
  return 0;
}

int gb_dirichlet_init(const gb_ctx *ctx, double *x) {
  if (!ctx || !x) return fail("NULL argument");
  const gb::Layout &L = ctx->c.L;
  for (int i = 0; i < L.N; i++)
    if (L.dbc[i]) x[i] = L.dbc_val[i];
  return 0;
}

int gb_matrix_fill_full_device(gb_ctx *ctx, const double *d_x, double *d_R, double *d_vals,
                               void *stream) {
  if (!ctx || !d_x || !d_R) return fail("NULL argument");
  return ctx->c.assemble(d_x, d_R, d_vals, (cudaStream_t)stream);
}

int gb_status(gb_ctx *ctx) {
  if (!ctx) return fail("NULL argument");
  return ctx->c.check_status();
}

int gb_matrix_fill_full(gb_ctx *ctx, const double *x, double *resid_vector, double *a_msr) {
  if (!ctx || !x || !resid_vector) return fail("NULL argument");
  Context &c = ctx->c;
  cudaError_t e = cudaMemcpyAsync(c.d_x, x, sizeof(double) * c.L.N, cudaMemcpyHostToDevice,
                                  c.stream);
  if (e != cudaSuccess) return cuda_fail(e, "x copy");
  if (c.assemble(c.d_x, c.d_R, a_msr ? c.d_vals : nullptr, c.stream)) return -1;
  e = cudaMemcpyAsync(resid_vector, c.d_R, sizeof(double) * c.L.N, cudaMemcpyDeviceToHost,
                      c.stream);
  if (e != cudaSuccess) return cuda_fail(e, "R copy");
  if (a_msr && c.to_msr_host(c.d_vals, a_msr)) return -1;
  return c.check_status();
}

int gb_device_buffers(gb_ctx *ctx, double **d_x, double **d_R, double **d_vals,
                      const long long **d_rowptr, const int **d_colidx) {
  if (!ctx) return fail("NULL argument");
  if (d_x) *d_x = ctx->c.d_x;
  if (d_R) *d_R = ctx->c.d_R;
  if (d_vals) *d_vals = ctx->c.d_vals;
  if (d_rowptr) *d_rowptr = (const long long *)ctx->c.d_rowptr;
  if (d_colidx) *d_colidx = ctx->c.d_colidx;
  return 0;
}

int gb_set_ilu_ordering(gb_ctx *ctx, int ordering) {
  if (!ctx || (ordering != GB_ILU_NATURAL && ordering != GB_ILU_MULTICOLOUR))
    return fail("ordering must be GB_ILU_NATURAL or GB_ILU_MULTICOLOUR");
  if (ctx->c.ilu_ordering != ordering) {
    ctx->c.ilu_ordering = ordering;
    ctx->c.solver.reset();  // rebuilt for the new order at the next solve
  }
  return 0;
}

int gb_set_element_density(gb_ctx *ctx, const double *rho) {
  if (!ctx) return fail("NULL argument");
  Context &c = ctx->c;
  if (!rho) {
    if (c.d_elem_rho) cudaFree(c.d_elem_rho);
    c.d_elem_rho = nullptr;
    return 0;
  }
  for (int e = 0; e < c.L.num_elems; e++)
    if (!(rho[e] > 0.0)) return fail("element densities must be positive");
  cudaError_t err = cudaSuccess;
  if (!c.d_elem_rho) err = cudaMalloc(&c.d_elem_rho, sizeof(double) * c.L.num_elems);
  if (err == cudaSuccess)
    err = cudaMemcpy(c.d_elem_rho, rho, sizeof(double) * c.L.num_elems, cudaMemcpyHostToDevice);
  return err == cudaSuccess ? 0 : cuda_fail(err, "element densities");
}

int gb_set_assembly_path(gb_ctx *ctx, int path) {
  if (!ctx || path < 0 || path > 4)
    return fail("path must be 0 (auto), 1 (scalar FP64), 2 (FP64 tensor pipe, per-fragment "
                "coefficients), 3 (FP64 tensor pipe, operand tables; 3-D Newtonian) or 4 (sum "
                "factorisation; 3-D Newtonian)");
  ctx->c.path = path;
  return 0;
}

int gb_set_triangular_solve(gb_ctx *ctx, int mode) {
  if (!ctx || mode < 0 || mode > 2)
    return fail("mode must be 0 (sync-free), 1 (level graph) or 2 (automatic)");
  ctx->c.trsv = mode;
  return 0;
}

int gb_set_sweep_fault(gb_ctx *ctx, long long spin_limit, int reverse_lower) {
  if (!ctx) return fail("NULL argument");
  ctx->c.sweep_spin_limit = spin_limit > 0 ? spin_limit : 0;
  ctx->c.sweep_reverse_lower = reverse_lower != 0;
  return 0;
}

int gb_set_material(gb_ctx *ctx, const gb_material *mat) {
  if (!ctx || !mat) return fail("NULL argument");
  return ctx->c.set_material(*mat);
}

int gb_kernel_timing(gb_ctx *ctx, int enable, double *kernel_ms, long long *launches) {
  if (!ctx) return fail("NULL argument");
  Context &c = ctx->c;
  if (kernel_ms) *kernel_ms = c.kernel_ms;
  if (launches) *launches = c.kernel_launches;
  if (enable && !c.ev_k0) {
    cudaEventCreate(&c.ev_k0);
    cudaEventCreate(&c.ev_k1);
  }
  c.timing = enable != 0;
  c.kernel_ms = 0.0;
  c.kernel_launches = 0;
  return 0;
}

void *gb_stream(gb_ctx *ctx) { return ctx ? (void *)ctx->c.stream : nullptr; }

int gb_csr_to_msr_host(gb_ctx *ctx, const double *d_vals, double *a_msr) {
  if (!ctx || !d_vals || !a_msr) return fail("NULL argument");
  return ctx->c.to_msr_host(d_vals, a_msr);
}

}  // extern "C"
