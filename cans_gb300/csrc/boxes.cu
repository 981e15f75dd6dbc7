// Batched time stepping of many independent boxes of uneven size (closed boxes /
// lid-driven cavities with implicit diffusion): one RK3 substep of every box is a fixed
// sequence of persistent launches over the concatenated work of all boxes --
//   momentum + RK update (mom_rk_cell), write-back with the implicit-diffusion correction,
//   the 3 x nbox velocity Helmholtz solves (one cans_batch), bounduvw, fillps,
//   updt_rhs_b + the nbox pressure solves (a second cans_batch), boundp, correc,
//   bounduvw, updatep, boundp
// -- and a whole time step (three substeps) can be captured once as a CUDA graph and
// replayed.  Each cell or face runs the same device body as the single-box kernels of
// stencil.cu, with the same arguments, so every box evolves bit-identically to the
// single-box call sequence of src/main.f90:452-472 (the order cans_gb300/driver.py uses).
//
// Scope: no flow-rate forcing (closed boxes), fixed dt per box (input dt_f), one GPU.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "bound_ops.h"
#include "stencil_body.cuh"

namespace {
constexpr int kTB = 256;
constexpr double kRk[3][2] = {{32. / 60., 0. / 60.}, {25. / 60., -17. / 60.}, {45. / 60., -25. / 60.}};

// per-box constants and device pointers of the cell kernels
struct BoxK {
  Dims d;
  int impdiff;
  double dxi, dyi, visc, bf[3];
  double f1[3], f2[3], f12[3];           // rk (src/rk.f90) per substep
  double dti[3], dtidxi[3], dtidyi[3];   // fillps with dti = 1/dtrk
  double cfi[3], cfj[3], cdt[3];         // correc with dt = dtrk
  double alpha[3];                       // updatep / Helmholtz alpha = -visc*dtrk/2
  const double *dzci, *dzfi;
  double *u, *v, *w, *p, *pp, *dudtrko, *dvdtrko, *dwdtrko, *unew, *dtd;
};

// one face task of a boundary call: a periodic halo copy or a set_bc on one face
struct FaceTask {
  double *p;
  int n1, n2, n3;
  int op;  // 0 set_bc, 1 halo copy
  int dir, ib, centered, up, lo;
  char ctype;
  double factor, sgn;
};

__device__ __forceinline__ int find_item(const long *__restrict__ start, int n, long w) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&start[mid]) <= w) lo = mid; else hi = mid - 1;
  }
  return lo;
}

enum CellOp { OP_MOM = 0, OP_WRITEBACK = 1, OP_FILLPS = 2, OP_CORREC = 3, OP_UPDATEP = 4 };

// persistent loop over 256-cell blocks of every box (start: per-box prefix of blocks)
template <int OP>
__global__ void __launch_bounds__(kTB) k_boxes_cells(const BoxK *__restrict__ box, const long *__restrict__ start,
                                                      int nbox, long total, int irk) {
  __shared__ double rdz[2 * 8];  // OP_MOM: the block's plane ratios (mom_rdz_table)
  for (long blk = blockIdx.x; blk < total; blk += gridDim.x) {
    const int s = find_item(start, nbox, blk);
    const BoxK &b = box[s];
    const long t0 = (blk - __ldg(&start[s])) * kTB, t = t0 + threadIdx.x;
    if (OP == OP_MOM) {
      const size_t np = (size_t)b.d.n1 * b.d.n2 * b.d.n3;
      int k0;
      const bool table = mom_rdz_table<8>(b.d, b.dzci, b.dzfi, rdz, k0, t0);
      mom_rk_cell<double>(b.d, b.dxi, b.dyi, b.visc, b.f1[irk], b.f2[irk], b.f12[irk], b.bf[0], b.bf[1], b.bf[2],
                          b.impdiff, b.dzci, b.dzfi, b.u, b.v, b.w, b.p, b.dudtrko, b.dvdtrko, b.dwdtrko, b.unew,
                          b.unew + np, b.unew + 2 * np, b.dtd, t, nullptr, 0., 0., 0., 0., table ? rdz : nullptr, k0);
      __syncthreads();  // the next block's table overwrites rdz
    } else if (OP == OP_WRITEBACK) {
      // rk.f90 write-back, then (implicit diffusion) u = (u - f12/2 dudtd) + f with f = 0
      // (no forcing): the expressions of k_rk_writeback and k_rk_forcing, fused
      int i, j, k;
      if (!cell3(t, b.d, i, j, k)) continue;
      const size_t np = (size_t)b.d.n1 * b.d.n2 * b.d.n3;
      const size_t c = hidx(i, j, k, b.d.n1, b.d.n2);
      double un = b.unew[t], vn = b.unew[t + np], wn = b.unew[t + 2 * np];
      if (b.impdiff) {
        const double f0 = 0., f12 = b.f12[irk];
        un = (un - .5 * f12 * b.dtd[t]) + f0;
        vn = (vn - .5 * f12 * b.dtd[t + np]) + f0;
        wn = (wn - .5 * f12 * b.dtd[t + 2 * np]) + f0;
      }
      b.u[c] = un; b.v[c] = vn; b.w[c] = wn;
    } else if (OP == OP_FILLPS) {
      fillps_cell(b.d, b.dti[irk], b.dtidxi[irk], b.dtidyi[irk], b.dzfi, b.u, b.v, b.w, b.pp, t);
    } else if (OP == OP_CORREC) {
      correc_cell(b.d, b.cfi[irk], b.cfj[irk], b.cdt[irk], b.dzci, b.pp, b.u, b.v, b.w, t);
    } else {
      updatep_cell(b.d, b.dxi, b.dyi, b.alpha[irk], b.impdiff, b.dzci, b.dzfi, b.pp, b.p, t);
    }
  }
}

__global__ void __launch_bounds__(kTB) k_boxes_faces(const FaceTask *__restrict__ task,
                                                      const long *__restrict__ start, int ntask, long total) {
  for (long blk = blockIdx.x; blk < total; blk += gridDim.x) {
    const int s = find_item(start, ntask, blk);
    const FaceTask &f = task[s];
    const long t = (blk - __ldg(&start[s])) * kTB + threadIdx.x;
    if (f.op == 0)
      set_bc_cell(f.p, f.n1, f.n2, f.n3, f.ctype, f.ib, f.dir, f.centered, f.factor, f.sgn, t);
    else
      halo_copy_cell(f.p, f.n1, f.n2, f.n3, f.dir, f.up, f.lo, t);
  }
}

// a device list of work items with its per-item prefix of 256-thread blocks
template <typename X> struct DevList {
  X *items = nullptr;
  long *start = nullptr;
  int n = 0;
  long total = 0;
  unsigned grid = 1;
};

// the face tasks of one boundary call, by phase: halo y, halo z, set_bc x, y, z
struct BoundCall {
  DevList<FaceTask> phase[5];
};

struct HostBox {
  cans_box in;
  double dl[3], dli[3];
  int is_bound[6];
  std::vector<double> dzc, dzf;  // host z grid (0:n3+1)
};
}  // namespace

struct cans_boxes {
  cudaStream_t stream;
  int nbox = 0, nsm = 0, impdiff = 1;
  std::vector<HostBox> hb;
  std::vector<cans_plan *> plans_v, plans_p;  // 3 per box (u, v, w), 1 per box
  cans_batch *bv = nullptr, *bp = nullptr;
  std::vector<double *> fv, fp;               // batch fields: u,v,w per box; pp per box
  std::vector<double> alpha_v[3];             // Helmholtz alpha per system and substep
  std::vector<int> isb_v, isb_p;
  double *scratch = nullptr;                  // unew + dtd of every box
  DevList<BoxK> cells, halo_cells;            // interior / haloed cell blocks
  BoundCall b_start_uvw, b_start_p, b_uvw_1, b_p_pp, b_uvw_2, b_p_p;
  std::vector<void *> allocs;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long graph_nodes = 0;
};

template <typename X>
static int upload_list(cans_boxes *B, const std::vector<X> &items, const std::vector<long> &blocks, DevList<X> &L) {
  L.n = (int)items.size();
  if (L.n == 0) return CANS_OK;
  std::vector<long> st(L.n + 1, 0);
  for (int e = 0; e < L.n; e++) st[e + 1] = st[e] + blocks[e];
  L.total = st[L.n];
  const size_t ib = sizeof(X) * L.n, sb = sizeof(long) * (L.n + 1);
  void *d = nullptr;
  CANS_CUDA_TRY(cudaMalloc(&d, ib + sb));
  B->allocs.push_back(d);
  CANS_CUDA_TRY(cudaMemcpy(d, items.data(), ib, cudaMemcpyHostToDevice));
  CANS_CUDA_TRY(cudaMemcpy((unsigned char *)d + ib, st.data(), sb, cudaMemcpyHostToDevice));
  L.items = (X *)d;
  L.start = (long *)((unsigned char *)d + ib);
  return CANS_OK;
}

static int grid_for(const void *fn, int nsm, long total, unsigned *grid) {
  int per = 0;
  CANS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kTB, 0));
  if (per < 1) return CANS_ENOTSUP;
  *grid = (unsigned)std::max(1L, std::min<long>(total, (long)per * nsm));
  return CANS_OK;
}

static long blocks_of(long cnt) { return (cnt + kTB - 1) / kTB; }

struct PhaseBuild {
  std::vector<FaceTask> t[5];
  std::vector<long> blk[5];
  // one face operation of a box's boundary call: phases halo y, halo z, set_bc x, y, z
  void add(const BcOp &o, double *p, const int n[3]) {
    FaceTask f;
    memset(&f, 0, sizeof(f));
    f.p = p; f.n1 = n[0]; f.n2 = n[1]; f.n3 = n[2];
    f.op = o.op; f.dir = o.dir; f.ib = o.ib; f.centered = o.centered; f.up = o.up; f.lo = o.lo;
    f.ctype = o.ctype; f.factor = o.factor; f.sgn = o.sgn;
    const int ph = o.op == 1 ? o.dir - 1 : 2 + o.dir;
    t[ph].push_back(f);
    blk[ph].push_back(blocks_of(bc_op_cells(o, n)));
  }
};

static void emit_bounduvw(PhaseBuild &pb, const HostBox &h, int keep_norm, int halos_norm, int halos_tang) {
  const cans_box &b = h.in;
  std::vector<BcOp> ops;
  bounduvw_ops(b.cbcvel, b.n, b.bcvel, h.is_bound, h.dl, h.dzc.data(), h.dzf.data(), keep_norm, halos_norm,
               halos_tang, ops);
  double *f[3] = {b.u, b.v, b.w};
  for (const BcOp &o : ops) pb.add(o, f[o.field], b.n);
}

static void emit_boundp(PhaseBuild &pb, const HostBox &h, double *p, int halo_side) {
  const cans_box &b = h.in;
  std::vector<BcOp> ops;
  boundp_ops(b.cbcpre, b.n, b.bcpre, h.is_bound, h.dl, h.dzc.data(), halo_side, ops);
  for (const BcOp &o : ops) pb.add(o, p, b.n);
}

static int finish_bound(cans_boxes *B, PhaseBuild &pb, BoundCall &bc) {
  for (int ph = 0; ph < 5; ph++) {
    int rc = upload_list(B, pb.t[ph], pb.blk[ph], bc.phase[ph]);
    if (rc) return rc;
    if (bc.phase[ph].n && (rc = grid_for((const void *)k_boxes_faces, B->nsm, bc.phase[ph].total, &bc.phase[ph].grid)))
      return rc;
  }
  return CANS_OK;
}

static int run_bound(cans_boxes *B, const BoundCall &bc) {
  for (int ph = 0; ph < 5; ph++) {
    const DevList<FaceTask> &L = bc.phase[ph];
    if (!L.n) continue;
    k_boxes_faces<<<L.grid, kTB, 0, B->stream>>>(L.items, L.start, L.n, L.total);
    CANS_LAUNCH_CHECK();
  }
  return CANS_OK;
}

extern "C" int cans_boxes_destroy(cans_boxes *B) {
  if (!B) return CANS_OK;
  if (B->exec) cudaGraphExecDestroy(B->exec);
  if (B->graph) cudaGraphDestroy(B->graph);
  cans_batch_destroy(B->bv);
  cans_batch_destroy(B->bp);
  for (auto p : B->plans_v) cans_plan_destroy(p);
  for (auto p : B->plans_p) cans_plan_destroy(p);
  for (auto a : B->allocs) cudaFree(a);
  cudaFree(B->scratch);
  delete B;
  return CANS_OK;
}

extern "C" int cans_boxes_create(int nbox, const cans_box *boxes, int is_impdiff, int autotune, void *stream,
                                 cans_boxes **out) {
  if (!out) return CANS_EINVAL;
  *out = nullptr;
  if (nbox < 1 || !boxes) return CANS_EINVAL;
  for (int s = 0; s < nbox; s++) {
    const cans_box &b = boxes[s];
    for (int d = 0; d < 3; d++) if (b.n[d] < 2 || !(b.l[d] > 0.)) return CANS_EINVAL;
    if (!(b.dt > 0.) || !b.dzc_g || !b.dzf_g || !b.dzci || !b.dzfi || !b.u || !b.v || !b.w || !b.p || !b.pp ||
        !b.dudtrko || !b.dvdtrko || !b.dwdtrko)
      return CANS_EINVAL;
    for (int e = 0; e < 18; e++) if (b.cbcvel[e] != 'P' && b.cbcvel[e] != 'D' && b.cbcvel[e] != 'N') return CANS_EINVAL;
    for (int e = 0; e < 6; e++) if (b.cbcpre[e] != 'P' && b.cbcpre[e] != 'D' && b.cbcpre[e] != 'N') return CANS_EINVAL;
  }
  cans_boxes *B = new cans_boxes();
  auto fail = [&](int rc) { cans_boxes_destroy(B); return rc; };
  B->stream = as_stream(stream);
  B->nbox = nbox;
  B->impdiff = is_impdiff ? 1 : 0;
  int dev = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&B->nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return fail(CANS_ECUDA);
  B->hb.resize(nbox);
  size_t scratch = 0;
  for (int s = 0; s < nbox; s++) {
    HostBox &h = B->hb[s];
    h.in = boxes[s];
    const cans_box &b = h.in;
    for (int d = 0; d < 3; d++) { h.dl[d] = b.l[d] / b.n[d]; h.dli[d] = 1. / h.dl[d]; }
    // is_bound on one GPU with x-aligned pencils (src/initmpi.f90:193-267)
    h.is_bound[0] = h.is_bound[1] = 1;
    for (int d = 1; d < 3; d++) {
      const int v = (b.cbcpre[2 * d] == 'P' && b.cbcpre[2 * d + 1] == 'P') ? 0 : 1;
      h.is_bound[2 * d] = h.is_bound[2 * d + 1] = v;
    }
    h.dzc.assign(b.dzc_g, b.dzc_g + b.n[2] + 2);
    h.dzf.assign(b.dzf_g, b.dzf_g + b.n[2] + 2);
    scratch += (size_t)(B->impdiff ? 6 : 3) * b.n[0] * b.n[1] * b.n[2];
  }
  {
    cudaError_t e = cudaMalloc(&B->scratch, scratch * sizeof(double));
    if (e != cudaSuccess) { cans_set_last_cuda_error(e); return fail(CANS_ENOMEM); }
  }
  // plans: velocity Helmholtz plans (face-centred along the component) and the pressure plan
  std::vector<BoxK> kb(nbox);
  std::vector<long> blk_in(nbox), blk_halo(nbox);
  size_t off = 0;
  for (int s = 0; s < nbox; s++) {
    HostBox &h = B->hb[s];
    const cans_box &b = h.in;
    const int n3 = b.n[2];
    std::vector<double> dzci_g(n3 + 2), dzfi_g(n3 + 2);
    for (int k = 0; k < n3 + 2; k++) { dzci_g[k] = 1. / h.dzc[k]; dzfi_g[k] = 1. / h.dzf[k]; }
    cans_plan *pl = nullptr;
    int rc;
    if (B->impdiff)
      for (int c = 0; c < 3; c++) {
        char cf[3] = {'c', 'c', 'c'};
        cf[c] = 'f';
        if ((rc = cans_initsolver(b.n, h.dli, dzci_g.data(), dzfi_g.data(), b.cbcvel + 6 * c, b.bcvel + 6 * c, cf,
                                  CANS_FP64, B->stream, &pl, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr)))
          return fail(rc);
        B->plans_v.push_back(pl);
      }
    const char ccc[3] = {'c', 'c', 'c'};
    if ((rc = cans_initsolver(b.n, h.dli, dzci_g.data(), dzfi_g.data(), b.cbcpre, b.bcpre, ccc, CANS_FP64, B->stream,
                              &pl, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr)))
      return fail(rc);
    B->plans_p.push_back(pl);
    // cell-kernel constants, evaluated as the single-box path does (driver.py / stencil.cu)
    BoxK &k = kb[s];
    memset(&k, 0, sizeof(k));
    k.d = Dims{b.n[0], b.n[1], b.n[2]};
    k.impdiff = B->impdiff;
    k.dxi = h.dli[0]; k.dyi = h.dli[1]; k.visc = b.visc;
    for (int d = 0; d < 3; d++) k.bf[d] = b.bforce[d];
    for (int irk = 0; irk < 3; irk++) {
      const double dt = b.dt;
      k.f1[irk] = kRk[irk][0] * dt;
      k.f2[irk] = kRk[irk][1] * dt;
      k.f12[irk] = k.f1[irk] + k.f2[irk];
      const double dtrk = (kRk[irk][0] + kRk[irk][1]) * dt, dtrki = 1. / dtrk;
      k.dti[irk] = dtrki; k.dtidxi[irk] = dtrki * h.dli[0]; k.dtidyi[irk] = dtrki * h.dli[1];
      k.cfi[irk] = dtrk * h.dli[0]; k.cfj[irk] = dtrk * h.dli[1]; k.cdt[irk] = dtrk;
      k.alpha[irk] = B->impdiff ? -.5 * b.visc * dtrk : 0.;
    }
    k.dzci = b.dzci; k.dzfi = b.dzfi;
    k.u = b.u; k.v = b.v; k.w = b.w; k.p = b.p; k.pp = b.pp;
    k.dudtrko = b.dudtrko; k.dvdtrko = b.dvdtrko; k.dwdtrko = b.dwdtrko;
    const size_t np = (size_t)b.n[0] * b.n[1] * b.n[2];
    k.unew = B->scratch + off;
    off += 3 * np;
    if (B->impdiff) { k.dtd = B->scratch + off; off += 3 * np; }
    blk_in[s] = blocks_of((long)np);
    blk_halo[s] = blocks_of((long)(b.n[0] + 2) * (b.n[1] + 2) * (b.n[2] + 2));
    if (B->impdiff) {
      B->fv.push_back(b.u); B->fv.push_back(b.v); B->fv.push_back(b.w);
      for (int irk = 0; irk < 3; irk++)
        for (int c = 0; c < 3; c++) B->alpha_v[irk].push_back(k.alpha[irk]);
      for (int c = 0; c < 3; c++) B->isb_v.insert(B->isb_v.end(), h.is_bound, h.is_bound + 6);
    }
    B->fp.push_back(b.pp);
    B->isb_p.insert(B->isb_p.end(), h.is_bound, h.is_bound + 6);
  }
  int rc;
  if (autotune) {
    // transform shapes are measured once per (length, kinds) and direction, on the largest
    // box that has it (most lines: least launch-latency bias), and reused for the others
    std::vector<int> order(nbox);
    for (int s = 0; s < nbox; s++) order[s] = s;
    std::sort(order.begin(), order.end(), [&](int a, int b) {
      const int *na = B->hb[a].in.n, *nb = B->hb[b].in.n;
      return (long)na[0] * na[1] * na[2] > (long)nb[0] * nb[1] * nb[2];
    });
    for (int s : order) {
      if ((rc = cans_plan_autotune(B->plans_p[s], 0, nullptr))) return fail(rc);
      if (B->impdiff)
        for (int c = 0; c < 3; c++)
          if ((rc = cans_plan_autotune(B->plans_v[3 * s + c], 0, nullptr))) return fail(rc);
    }
  }
  if ((rc = upload_list(B, kb, blk_in, B->cells)) || (rc = upload_list(B, kb, blk_halo, B->halo_cells))) return fail(rc);
  if ((rc = grid_for((const void *)k_boxes_cells<OP_MOM>, B->nsm, B->cells.total, &B->cells.grid)) ||
      (rc = grid_for((const void *)k_boxes_cells<OP_CORREC>, B->nsm, B->halo_cells.total, &B->halo_cells.grid)))
    return fail(rc);
  if (B->impdiff && (rc = cans_batch_create((int)B->plans_v.size(), B->plans_v.data(), B->stream, &B->bv)))
    return fail(rc);
  if ((rc = cans_batch_create((int)B->plans_p.size(), B->plans_p.data(), B->stream, &B->bp))) return fail(rc);
  // boundary calls of the time loop (src/main.f90:388-418, 452-472)
  {
    PhaseBuild a, c, d, e, f, g;
    for (auto &h : B->hb) {
      emit_bounduvw(a, h, 0, 2, 2);
      emit_boundp(c, h, h.in.p, 1);
      emit_bounduvw(d, h, 0, -1, 2);
      emit_boundp(e, h, h.in.pp, 2);
      emit_bounduvw(f, h, 1, 1, 0);
      emit_boundp(g, h, h.in.p, 1);
    }
    if ((rc = finish_bound(B, a, B->b_start_uvw)) || (rc = finish_bound(B, c, B->b_start_p)) ||
        (rc = finish_bound(B, d, B->b_uvw_1)) || (rc = finish_bound(B, e, B->b_p_pp)) ||
        (rc = finish_bound(B, f, B->b_uvw_2)) || (rc = finish_bound(B, g, B->b_p_p)))
      return fail(rc);
  }
  *out = B;
  return CANS_OK;
}

// boundary conditions on the initial fields (src/main.f90:388-418)
extern "C" int cans_boxes_start(cans_boxes *B) {
  if (!B) return CANS_EINVAL;
  int rc;
  if ((rc = run_bound(B, B->b_start_uvw)) || (rc = run_bound(B, B->b_start_p))) return rc;
  return CANS_OK;
}

template <int OP> static int run_cells(cans_boxes *B, const DevList<BoxK> &L, int irk) {
  k_boxes_cells<OP><<<L.grid, kTB, 0, B->stream>>>(L.items, L.start, L.n, L.total, irk);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

extern "C" int cans_boxes_substep(cans_boxes *B, int irk) {
  if (!B || irk < 0 || irk > 2) return CANS_EINVAL;
  int rc;
  if ((rc = run_cells<OP_MOM>(B, B->cells, irk)) || (rc = run_cells<OP_WRITEBACK>(B, B->cells, irk))) return rc;
  if (B->impdiff && (rc = cans_batch_solve(B->bv, B->fv.data(), B->alpha_v[irk].data(), B->isb_v.data()))) return rc;
  if ((rc = run_bound(B, B->b_uvw_1))) return rc;
  if ((rc = run_cells<OP_FILLPS>(B, B->cells, irk))) return rc;
  if ((rc = cans_batch_solve(B->bp, B->fp.data(), nullptr, B->isb_p.data()))) return rc;
  if ((rc = run_bound(B, B->b_p_pp))) return rc;
  if ((rc = run_cells<OP_CORREC>(B, B->halo_cells, irk))) return rc;
  if ((rc = run_bound(B, B->b_uvw_2))) return rc;
  if ((rc = run_cells<OP_UPDATEP>(B, B->cells, irk))) return rc;
  if ((rc = run_bound(B, B->b_p_p))) return rc;
  return CANS_OK;
}

static int enqueue_step(cans_boxes *B) {
  for (int irk = 0; irk < 3; irk++) {
    int rc = cans_boxes_substep(B, irk);
    if (rc) return rc;
  }
  return CANS_OK;
}

// one time step (three substeps).  use_graph: the first call runs the step eagerly (building
// the solve work tables and factorisations), the second captures it as a CUDA graph, and
// every later call replays the graph with one launch.
extern "C" int cans_boxes_step(cans_boxes *B, int use_graph) {
  if (!B) return CANS_EINVAL;
  if (!use_graph) return enqueue_step(B);
  if (B->exec) {
    CANS_CUDA_TRY(cudaGraphLaunch(B->exec, B->stream));
    cans_count_launch();
    return CANS_OK;
  }
  if (!B->stream) return CANS_EINVAL;  // the legacy default stream cannot be captured
  if (!B->graph) {
    // warm-up step: work tables and factorisations exist before capture
    int rc = enqueue_step(B);
    if (rc) return rc;
    CANS_CUDA_TRY(cudaStreamSynchronize(B->stream));
    CANS_CUDA_TRY(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
    rc = enqueue_step(B);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(B->stream, &g);
    if (rc || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (e != cudaSuccess) cans_set_last_cuda_error(e);
      return rc ? rc : CANS_ECUDA;
    }
    B->graph = g;
    size_t nn = 0;
    cudaGraphGetNodes(g, nullptr, &nn);
    B->graph_nodes = (long long)nn;
    CANS_CUDA_TRY(cudaGraphInstantiate(&B->exec, g, 0));
    return CANS_OK;  // the warm-up step was this call's step
  }
  return CANS_OK;
}

extern "C" long long cans_boxes_graph_nodes(const cans_boxes *B) { return B ? B->graph_nodes : 0; }
