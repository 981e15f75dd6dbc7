// Boundary-condition calls as ordered lists of face operations (host side), shared by the
// single-box launches (stencil.cu), the batched boxes (boxes.cu) and the adjoints
// (adjoint.cu).  The order is the CPU path's of src/bound.f90:17-180 on one GPU with
// x-aligned pencils: periodic y/z ghosts that are not a domain bound are local copies,
// then set_bc per direction, side and component.
#pragma once
#include <vector>

struct BcOp {
  int field;      // 0, 1, 2: u, v, w (bounduvw); 0: p (boundp)
  int op;         // 0 set_bc, 1 periodic halo copy
  int dir, ib, centered, up, lo;
  char ctype;
  double factor, sgn;
};

// set_bc's ghost formula coefficients (src/bound.f90:182-463, nh = 1)
inline BcOp bc_op(int field, char ctype, int ib, int dir, int centered, double rvalue, double dr) {
  BcOp o{};
  double factor = rvalue, sgn = 0.;
  if (ctype == 'D' && centered) { factor = 2. * factor; sgn = -1.; }
  if (ctype == 'N') { factor = ib == 0 ? -dr * factor : dr * factor; sgn = 1.; }
  o.field = field; o.op = 0; o.ctype = ctype; o.ib = ib; o.dir = dir; o.centered = centered;
  o.factor = factor; o.sgn = sgn;
  return o;
}

inline bool halo_op(int field, int dir, int side, BcOp *o) {
  const int up = side == 2 || side == 1, lo = side == 2 || side == -1;
  if (!(up || lo)) return false;
  *o = BcOp{};
  o->field = field; o->op = 1; o->dir = dir; o->up = up; o->lo = lo;
  return true;
}

// bounduvw (src/bound.f90:17-122); halos_*: -1 lower, 0 none, 1 upper, 2 both
inline void bounduvw_ops(const char cbc[18], const int n[3], const double bc[18], const int is_bound[6],
                         const double dl[3], const double *dzc, const double *dzf, int keep_norm, int halos_norm,
                         int halos_tang, std::vector<BcOp> &out) {
  int updt_norm[2] = {1, 1};
  if (halos_norm == -1) updt_norm[1] = 0;
  else if (halos_norm == 0) updt_norm[0] = updt_norm[1] = 0;
  else if (halos_norm == 1) updt_norm[0] = 0;
  for (int dd = 1; dd < 3; dd++)
    for (int c = 0; c < 3; c++) {
      const bool pp = cbc[2 * dd + 6 * c] == 'P' && cbc[1 + 2 * dd + 6 * c] == 'P';
      if (!pp || is_bound[2 * dd] || is_bound[2 * dd + 1]) continue;
      BcOp o;
      if (halo_op(c, dd, c == dd ? halos_norm : halos_tang, &o)) out.push_back(o);
    }
  for (int dd = 0; dd < 3; dd++)
    for (int ib = 0; ib < 2; ib++) {
      if (!is_bound[ib + 2 * dd]) continue;
      const bool pp = cbc[2 * dd + 6 * dd] == 'P' && cbc[1 + 2 * dd + 6 * dd] == 'P';
      const bool apply_norm = !keep_norm || (pp && updt_norm[ib]);
      for (int c = 0; c < 3; c++) {
        double dr;
        if (dd < 2) dr = dl[dd];
        else if (c == 2) dr = ib == 0 ? dzf[0] : dzf[n[2]];
        else dr = ib == 0 ? dzc[0] : dzc[n[2]];
        const char ct = cbc[ib + 2 * dd + 6 * c];
        const double bv = bc[ib + 2 * dd + 6 * c];
        if (c == dd) {
          if (apply_norm) out.push_back(bc_op(c, ct, ib, dd, 0, bv, dr));
        } else {
          out.push_back(bc_op(c, ct, ib, dd, 1, bv, dr));
        }
      }
    }
}

// boundp (src/bound.f90:124-180); halo_side: -1 lower, 0 none, 1 upper, 2 both
inline void boundp_ops(const char cbc[6], const int n[3], const double bc[6], const int is_bound[6],
                       const double dl[3], const double *dzc, int halo_side, std::vector<BcOp> &out) {
  int upd[2] = {1, 1};
  if (halo_side == -1) upd[1] = 0;
  else if (halo_side == 0) upd[0] = upd[1] = 0;
  else if (halo_side == 1) upd[0] = 0;
  for (int dd = 1; dd < 3; dd++) {
    const bool pp = cbc[2 * dd] == 'P' && cbc[2 * dd + 1] == 'P';
    if (!pp || is_bound[2 * dd] || is_bound[2 * dd + 1]) continue;
    BcOp o;
    if (halo_op(0, dd, halo_side, &o)) out.push_back(o);
  }
  for (int dd = 0; dd < 3; dd++)
    for (int ib = 0; ib < 2; ib++) {
      if (!is_bound[ib + 2 * dd] || !upd[ib]) continue;
      const double dr = dd < 2 ? dl[dd] : (ib == 0 ? dzc[0] : dzc[n[2]]);
      out.push_back(bc_op(0, cbc[ib + 2 * dd], ib, dd, 1, bc[ib + 2 * dd], dr));
    }
}

// cells of one face operation's launch: set_bc covers the haloed extent of the two other
// directions; a halo copy covers x (haloed) times the other periodic-plane direction
inline long bc_op_cells(const BcOp &o, const int n[3]) {
  if (o.op == 0) return (long)((o.dir == 0 ? n[1] : n[0]) + 2) * ((o.dir == 2 ? n[1] : n[2]) + 2);
  return (long)(n[0] + 2) * ((o.dir == 1 ? n[2] : n[1]) + 2);
}
