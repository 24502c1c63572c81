/*
 * rich_oracle.c -- CPU restatement of RICH's hydro hot path (parity oracle).
 *
 * TEST INFRASTRUCTURE ONLY (see rich_oracle.h).  Build with
 *   gcc -O2 -ffp-contract=off -fPIC -shared rich_oracle.c -lm
 * so that no multiply-add is contracted; the reference fixtures are built
 * the same way.
 *
 * Paths are relative to the RICH source root (source/...).  Each function
 * follows the reference expression by expression; comments give the file and
 * lines.  Vector2D / ComputationalCell arithmetic is expanded component-wise
 * with the same operands in the same order (tessellation/geometry.cpp,
 * two_dimensional/computational_cell_2d.cpp, common/hydrodynamic_variables.cpp).
 */
#include "rich_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* M_PI as <cmath> defines it for the reference (VoronoiMesh.cpp:412) */
#define RO_PI 3.14159265358979323846

typedef struct { double x, y; } v2;
typedef struct { double d, p, vx, vy; } cc;           /* ComputationalCell (no tracers) */
typedef struct { double d, p, vx, vy, e, c; } prim;   /* Primitive */
typedef struct { double m, mx, my, en; } cons;        /* Conserved */

/* std::min / std::max: min(a,b) = b<a ? b : a; max(a,b) = a<b ? b : a. */
static double smin(double a, double b) { return b < a ? b : a; }
static double smax(double a, double b) { return a < b ? b : a; }
/* geometry.cpp:18-21 abs(Vector2D) */
static double vabs(v2 v) { return sqrt(v.x * v.x + v.y * v.y); }
/* geometry.cpp:100-105 ScalarProd */
static double dot(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
static v2 vsub(v2 a, v2 b) { v2 r = {a.x - b.x, a.y - b.y}; return r; }
static v2 vadd(v2 a, v2 b) { v2 r = {a.x + b.x, a.y + b.y}; return r; }
/* geometry.cpp:85-93 d*v and v*d both give (v.x*d, v.y*d) */
static v2 vscale(v2 v, double d) { v2 r = {v.x * d, v.y * d}; return r; }
/* geometry.cpp:95-98 */
static v2 vdiv(v2 v, double d) { v2 r = {v.x / d, v.y / d}; return r; }

static v2 point(const rg_mesh_view* m, int i) { v2 r = {m->point_xy[2 * i], m->point_xy[2 * i + 1]}; return r; }
static v2 cmof(const rg_mesh_view* m, int i) { v2 r = {m->cm_xy[2 * i], m->cm_xy[2 * i + 1]}; return r; }
static v2 vert0(const rg_mesh_view* m, int e) { v2 r = {m->face_vertices[4 * e], m->face_vertices[4 * e + 1]}; return r; }
static v2 vert1(const rg_mesh_view* m, int e) { v2 r = {m->face_vertices[4 * e + 2], m->face_vertices[4 * e + 3]}; return r; }
static int fc0(const rg_mesh_view* m, int e) { return m->face_cells[2 * e]; }
static int fc1(const rg_mesh_view* m, int e) { return m->face_cells[2 * e + 1]; }
/* VoronoiMesh.cpp:169-206 GetOriginalIndex */
static int orig(const rg_mesh_view* m, int p) { return p < m->n_cells ? p : m->ghost_source[p - m->n_cells]; }
static cc cell_at(const double* cells, int i) { cc r = {cells[4 * i], cells[4 * i + 1], cells[4 * i + 2], cells[4 * i + 3]}; return r; }

static void set_err(ro_error* err, int status, int phase, int64_t index, double value) {
  if (err && err->status == 0) {
    err->status = status;
    err->phase = phase;
    err->index = index;
    err->value = value;
  }
}

/* spatial_reconstruction.cpp:3-6 CalcCentroid: 0.5*(first+second) */
static v2 centroid(const rg_mesh_view* m, int e) { return vscale(vadd(vert0(m, e), vert1(m, e)), 0.5); }
/* Edge.cpp:83-86 Parallel: second - first */
static v2 parallel(const rg_mesh_view* m, int e) { return vsub(vert1(m, e), vert0(m, e)); }
/* Edge.cpp GetLength: abs(second-first); physical_geometry.cpp:8-11 calcArea: abs(first-second) */
static double edge_length(const rg_mesh_view* m, int e) { return vabs(vsub(vert1(m, e), vert0(m, e))); }
static double edge_area(const rg_mesh_view* m, int e) { return vabs(vsub(vert0(m, e), vert1(m, e))); }
/* VoronoiMesh.cpp:410-413 GetWidth */
static double width(const rg_mesh_view* m, int i) { return sqrt(m->volume[i] / RO_PI); }

/* ideal_gas.cpp:13-16 dp2e, :40-44 dp2c, :18-23 de2p */
static double dp2e(double g, double d, double p) { return p / d / (g - 1); }
static double dp2c(double g, double d, double p) { return sqrt(g * p / d); }

/* simple_flux_calculator.cpp:9-15 convert_to_primitive */
static prim to_prim(double g, cc c) {
  prim r;
  r.d = c.d;
  r.p = c.p;
  r.vx = c.vx;
  r.vy = c.vy;
  r.e = dp2e(g, c.d, c.p);
  r.c = dp2c(g, c.d, c.p);
  return r;
}

/* simple_flux_calculator.cpp:17-25 reflect, geometry.cpp:117-120 Reflect:
 * 2*ScalarProd(v,axis)*axis/pow(abs(axis),2)-v (pow(x,2) folds to x*x). */
static prim reflect(prim p, v2 axis) {
  v2 v = {p.vx, p.vy};
  const double s = 2 * dot(v, axis);
  const double aa = vabs(axis);
  const v2 t = vdiv(vscale(axis, s), aa * aa);
  p.vx = t.x - v.x;
  p.vy = t.y - v.y;
  return p;
}

/* hydrodynamic_variables.cpp:261-265 TotalEnergyDensity: d*(0.5*pow(abs(v),2)+e) */
static double ted(prim p) {
  v2 v = {p.vx, p.vy};
  const double s = vabs(v);
  return p.d * (0.5 * (s * s) + p.e);
}

/* hydrodynamic_variables.cpp:267-272 Primitive2Conserved */
static cons p2c(prim p) {
  cons r;
  r.m = p.d;
  r.mx = p.vx * p.d;
  r.my = p.vy * p.d;
  r.en = ted(p);
  return r;
}

/* hydrodynamic_variables.cpp:281-290 Primitive2Flux with n = (1,0) */
static cons p2f_x(prim p) {
  const v2 n = {1, 0};
  const v2 nn = vdiv(n, vabs(n));
  const v2 v = {p.vx, p.vy};
  const double sp = dot(v, nn);
  cons r;
  r.m = p.d * sp;
  const double dsp = p.d * sp;
  r.mx = nn.x * p.p + v.x * dsp;
  r.my = nn.y * p.p + v.y * dsp;
  r.en = (ted(p) + p.p) * sp;
  return r;
}

/* hllc.cpp:76-92 starred_state */
static cons starred(prim s, double sk, double ss) {
  const double dk = s.d, pk = s.p, uk = s.vx, vk = s.vy;
  const double ds = dk * (sk - uk) / (sk - ss);
  const double ek = ted(s);
  cons r;
  r.m = ds;
  r.mx = ds * ss;
  r.my = ds * vk;
  r.en = ek * ds / dk + ds * (ss - uk) * (ss + pk / dk / (sk - uk));
  return r;
}

/* hllc.cpp:97-154 Hllc::operator() with massflux_ = true */
static int hllc(prim left, prim right, double velocity, cons* out, int64_t face, ro_error* err) {
  if (isnan(right.vx)) {
    set_err(err, RG_ERR_HLLC_NAN, 3, face, right.vx);
    return RG_ERR_HLLC_NAN;
  }
  /* local.Velocity -= velocity*normaldir, normaldir = (1,0) */
  const double bx = 1 * velocity, by = 0 * velocity;
  left.vx -= bx;
  left.vy -= by;
  right.vx -= bx;
  right.vy -= by;
  /* hllc.cpp:27-43 estimate_wave_speeds */
  const double dl = left.d, pl = left.p, vl = left.vx, cl = left.c;
  const double dr = right.d, pr = right.p, vr = right.vx, cr = right.c;
  const double sl = smin(vl - cl, vr - cr);
  const double sr = smax(vl + cl, vr + cr);
  const double ss = (pr - pl + dl * vl * (sl - vl) - dr * vr * (sr - vr)) / (dl * (sl - vl) - dr * (sr - vr));
  const cons ul = p2c(left), ur = p2c(right);
  const cons fl = p2f_x(left), fr = p2f_x(right);
  const cons usl = starred(left, sl, ss), usr = starred(right, sr, ss);
  cons f;
  if (sl > 0)
    f = fl;
  else if (sl <= 0 && ss >= 0) {
    f.m = fl.m + sl * (usl.m - ul.m);
    f.mx = fl.mx + (usl.mx - ul.mx) * sl;
    f.my = fl.my + (usl.my - ul.my) * sl;
    f.en = fl.en + sl * (usl.en - ul.en);
  } else if (ss < 0 && sr >= 0) {
    f.m = fr.m + sr * (usr.m - ur.m);
    f.mx = fr.mx + (usr.mx - ur.mx) * sr;
    f.my = fr.my + (usr.my - ur.my) * sr;
    f.en = fr.en + sr * (usr.en - ur.en);
  } else if (sr < 0)
    f = fr;
  else {
    set_err(err, RG_ERR_HLLC_WAVE_SPEEDS, 3, face, ss);
    return RG_ERR_HLLC_WAVE_SPEEDS;
  }
  /* hllc.cpp:150-152 */
  const v2 vn = {1 * velocity, 0 * velocity};
  const v2 mom = {f.mx, f.my};
  f.en += dot(mom, vn) + 0.5 * f.m * velocity * velocity;
  const double vm = velocity * f.m;
  f.mx += 1 * vm;
  f.my += 0 * vm;
  *out = f;
  return 0;
}

/* LagrangianHLLC.cpp:85-175 LagrangianHLLC::operator(): Hllc's flux, with
 * massflux = 0 taken in the frame of the contact (estimate_wave_speeds of the
 * boosted states), and the transferred internal energy `energy` (the
 * contact speed when massflux = 0) */
static int lhllc(prim left, prim right, double velocity, int massflux, cons* out, double* energy, int64_t face,
                 ro_error* err) {
  if (isnan(right.vx)) {
    set_err(err, RG_ERR_HLLC_NAN, 3, face, right.vx);
    return RG_ERR_HLLC_NAN;
  }
  const double bx = 1 * velocity, by = 0 * velocity;
  left.vx -= bx;
  left.vy -= by;
  right.vx -= bx;
  right.vy -= by;
  double en = 0;
  if (!massflux) {
    const double sl2 = smin(left.vx - left.c, right.vx - right.c);
    const double sr2 = smax(left.vx + left.c, right.vx + right.c);
    const double ss2 = (right.p - left.p + left.d * left.vx * (sl2 - left.vx) - right.d * right.vx * (sr2 - right.vx)) /
                       (left.d * (sl2 - left.vx) - right.d * (sr2 - right.vx));
    const double cx = ss2 * 1, cy = ss2 * 0;
    left.vx -= cx;
    left.vy -= cy;
    right.vx -= cx;
    right.vy -= cy;
    velocity += ss2;
    en = ss2;
  }
  const double dl = left.d, pl = left.p, vl = left.vx, cl = left.c;
  const double dr = right.d, pr = right.p, vr = right.vx, cr = right.c;
  const double sl = smin(vl - cl, vr - cr);
  const double sr = smax(vl + cl, vr + cr);
  const double ss = (pr - pl + dl * vl * (sl - vl) - dr * vr * (sr - vr)) / (dl * (sl - vl) - dr * (sr - vr));
  const cons ul = p2c(left), ur = p2c(right);
  const cons fl = p2f_x(left), fr = p2f_x(right);
  const cons usl = starred(left, sl, ss), usr = starred(right, sr, ss);
  const v2 xdir = {1, 0};
  const v2 vlv = {left.vx, left.vy}, vrv = {right.vx, right.vy};
  cons f;
  if (sl > 0) {
    f = fl;
    if (massflux) en = dot(vlv, xdir) * left.e * left.d;
  } else if (sl <= 0 && ss >= 0) {
    f.m = fl.m + sl * (usl.m - ul.m);
    f.mx = fl.mx + (usl.mx - ul.mx) * sl;
    f.my = fl.my + (usl.my - ul.my) * sl;
    f.en = fl.en + sl * (usl.en - ul.en);
    if (massflux)
      en = dot(vlv, xdir) * left.e * left.d + sl * left.e * ((sl - left.vx) / (sl - ss) - 1) * left.d;
  } else if (ss < 0 && sr >= 0) {
    f.m = fr.m + sr * (usr.m - ur.m);
    f.mx = fr.mx + (usr.mx - ur.mx) * sr;
    f.my = fr.my + (usr.my - ur.my) * sr;
    f.en = fr.en + sr * (usr.en - ur.en);
    if (massflux) en = (dot(vrv, xdir) * right.e + sr * right.e * ((sr - right.vx) / (sr - ss) - 1)) * right.d;
  } else if (sr < 0) {
    f = fr;
    if (massflux) en = dot(vrv, xdir) * right.e * right.d;
  } else {
    set_err(err, RG_ERR_HLLC_WAVE_SPEEDS, 3, face, ss);
    return RG_ERR_HLLC_WAVE_SPEEDS;
  }
  const v2 vn = {1 * velocity, 0 * velocity};
  const v2 mom = {f.mx, f.my};
  f.en += dot(mom, vn) + 0.5 * f.m * velocity * velocity;
  const double vm = velocity * f.m;
  f.mx += 1 * vm;
  f.my += 0 * vm;
  *out = f;
  *energy = en;
  return 0;
}

/* simple_flux_calculator.cpp:130-140 rotate: (Projection(v,n), Projection(v,p)) */
static prim rotate(prim s, v2 n, v2 p) {
  const v2 v = {s.vx, s.vy};
  s.vx = dot(v, n) / vabs(n);
  s.vy = dot(v, p) / vabs(p);
  return s;
}

/* simple_flux_calculator.cpp:142-165 rotate_back / rotate_solve_rotate_back */
static int rotate_solve_rotate_back(prim left, prim right, double velocity, v2 n, v2 p, cons* out,
                                    int64_t face, ro_error* err) {
  cons c;
  const int st = hllc(rotate(left, n, p), rotate(right, n, p), velocity, &c, face, err);
  if (st) return st;
  const v2 a = vdiv(vscale(n, c.mx), vabs(n));
  const v2 b = vdiv(vscale(p, c.my), vabs(p));
  out->m = c.m;
  out->mx = a.x + b.x;
  out->my = a.y + b.y;
  out->en = c.en;
  return 0;
}

static void put_flux(double* f, cons c) { f[0] = c.m; f[1] = c.en; f[2] = c.mx; f[3] = c.my; }

/* rotate_solve_rotate_back with LagrangianHLLC (LagrangianFlux, condition_action_sequence_2.cpp:284-290) */
static int rotate_solve_rotate_back_lag(prim left, prim right, double velocity, int massflux, v2 n, v2 p, cons* out,
                                        double* energy, int64_t face, ro_error* err) {
  cons c;
  const int st = lhllc(rotate(left, n, p), rotate(right, n, p), velocity, massflux, &c, energy, face, err);
  if (st) return st;
  const v2 a = vdiv(vscale(n, c.mx), vabs(n));
  const v2 b = vdiv(vscale(p, c.my), vabs(p));
  out->m = c.m;
  out->mx = a.x + b.x;
  out->my = a.y + b.y;
  out->en = c.en;
  return 0;
}

/* State of a point (real cell or ghost) as SimpleFluxCalculator sees it:
 * a ghost that is not a self-mirror takes its source cell's state (the
 * reference indexes cells[] with the ghost id there, which only exists in
 * MPI builds; the source cell is what that entry holds). */
static cc point_state(const rg_mesh_view* m, const double* cells, int p) {
  return cell_at(cells, orig(m, p));
}

/* simple_flux_calculator.cpp:80-126 riemann_reduce + :167-189 calcHydroFlux
 * + :216-244 operator() */
int ro_simple_flux(const rg_mesh_view* m, const double* cells, const double* ev, double g,
                   double* fluxes, ro_error* err) {
  const int N = m->n_cells;
  for (int e = 0; e < m->n_faces; ++e) {
    const int a = fc0(m, e), b = fc1(m, e);
    const v2 p = parallel(m, e);
    const v2 n = vsub(point(m, b), point(m, a));
    const int va = a >= 0 && a < N, vb = b >= 0 && b < N;
    prim left, right;
    if (!va) {
      right = to_prim(g, point_state(m, cells, b));
      if (orig(m, b) == orig(m, a))
        left = reflect(right, p);
      else
        left = to_prim(g, point_state(m, cells, a));
    } else if (!vb) {
      left = to_prim(g, point_state(m, cells, a));
      if (orig(m, b) == orig(m, a))
        right = reflect(left, p);
      else
        right = to_prim(g, point_state(m, cells, b));
    } else {
      left = to_prim(g, cell_at(cells, a));
      right = to_prim(g, cell_at(cells, b));
    }
    const v2 w = {ev[2 * e], ev[2 * e + 1]};
    const double velocity = dot(n, w) / vabs(n);
    cons c;
    const int st = rotate_solve_rotate_back(left, right, velocity, n, p, &c, e, err);
    if (st) return st;
    put_flux(fluxes + 4 * e, c);
  }
  return 0;
}

/* ---------------- LinearGaussImproved (interpolations/LinearGaussImproved.cpp) ---------- */

/* computational_cell_2d.cpp:59-68 ComputationalCellAddMult */
static void addmult(cc* r, cc o, double s) {
  r->d += o.d * s;
  r->p += o.p * s;
  r->vx += o.vx * s;
  r->vy += o.vy * s;
}
static cc ccsub(cc a, cc b) { cc r = {a.d - b.d, a.p - b.p, a.vx - b.vx, a.vy - b.vy}; return r; }
static cc ccscale(cc a, double s) { cc r = {a.d * s, a.p * s, a.vx * s, a.vy * s}; return r; }
static cc ccadd(cc a, cc b) { cc r = {a.d + b.d, a.p + b.p, a.vx + b.vx, a.vy + b.vy}; return r; }

typedef struct { cc x, y; } slope;

/* Tracers of one cell and of its neighbours during LinearGaussImproved
 * (ComputationalCell::tracers, computational_cell_2d.hpp): every
 * ComputationalCell operation above applies to each tracer exactly as to a
 * hydro field, so the tracer parts run beside the hydro ones with the same
 * scalars. */
#define RO_MAX_NB 64
typedef struct {
  int nt;
  double ct[RG_MAX_TRACERS];              /* the cell's tracers */
  double nb[RO_MAX_NB][RG_MAX_TRACERS];   /* neighbours' tracers (ghosts: copied cell's) */
  double sx[RG_MAX_TRACERS], sy[RG_MAX_TRACERS];  /* tracer slopes */
} trcell;

/* Ghost states: RigidWallGenerator.cpp:17-37 / PeriodicGhostGenerator.cpp:3-17.
 * new_cells[ghost] for every ghost (LinearGaussImproved.cpp:543-550). */
static void ghost_states(const rg_mesh_view* m, const double* cells, int ghost_kind, cc* gs) {
  const int N = m->n_cells;
  for (int g = 0; g < m->n_ghosts; ++g) {
    const int e = m->ghost_face[g];
    memset(&gs[g], 0, sizeof(cc));
    if (e < 0) continue;
    const int a = fc0(m, e), b = fc1(m, e);
    if (ghost_kind == RG_GHOST_PERIODIC) {
      gs[g] = cell_at(cells, m->ghost_source[g]);
    } else {
      /* index 1: ghost is neighbors.first; the real side is the other one */
      const int ghost_first = a >= N;
      const int real = ghost_first ? b : a;
      cc c = cell_at(cells, real);
      /* RigidWallGenerator.cpp:5-15 ReverseNormalVelocity */
      v2 normal = ghost_first ? vsub(point(m, a), point(m, b)) : vsub(point(m, b), point(m, a));
      normal = vdiv(normal, vabs(normal));
      const v2 v = {c.vx, c.vy};
      const v2 t = vscale(normal, 2 * dot(v, normal));
      c.vx -= t.x;
      c.vy -= t.y;
      gs[g] = c;
    }
  }
}

static cc any_state(const rg_mesh_view* m, const double* cells, const cc* gs, int p) {
  return p < m->n_cells ? cell_at(cells, p) : gs[p - m->n_cells];
}

/* :159-165 interp and :167-172 interp2 */
static void interp2(cc* r, slope s, v2 target, v2 cm) {
  addmult(r, s.x, target.x - cm.x);
  addmult(r, s.y, target.y - cm.y);
}

/* :67-134 calc_naive_slope */
static int naive_slope(const rg_mesh_view* m, int i, cc cell, v2 center, v2 cell_cm, double vol,
                       const int* edges, int n, const cc* nb, const v2* nb_pt, const v2* nb_cm,
                       slope* res, trcell* t, ro_error* err) {
  if (n > 20) {
    set_err(err, RG_ERR_TOO_MANY_NEIGHBORS, 2, i, n);
    return RG_ERR_TOO_MANY_NEIGHBORS;
  }
  double mm[4] = {0, 0, 0, 0};
  slope vc = {{0, 0, 0, 0}, {0, 0, 0, 0}};
  double tvx[RG_MAX_TRACERS], tvy[RG_MAX_TRACERS];
  const int nt = t ? t->nt : 0;
  for (int k = 0; k < n; ++k) {
    const int e = edges[k];
    const v2 c_ij = vsub(centroid(m, e), vscale(vadd(nb_cm[k], cell_cm), 0.5));
    const double e_length = edge_length(m, e);
    const v2 dd = vsub(nb_pt[k], center);
    const v2 r_ij = vscale(vdiv(dd, vabs(dd)), e_length);
    mm[0] -= c_ij.x * r_ij.x;
    mm[1] -= c_ij.y * r_ij.x;
    mm[2] -= c_ij.x * r_ij.y;
    mm[3] -= c_ij.y * r_ij.y;
    if (k == 0) {
      vc.x = ccscale(cell, r_ij.x * 0.5);
      vc.y = ccscale(cell, r_ij.y * 0.5);
    } else {
      addmult(&vc.x, cell, r_ij.x * 0.5);
      addmult(&vc.y, cell, r_ij.y * 0.5);
    }
    addmult(&vc.y, nb[k], r_ij.y * 0.5);
    addmult(&vc.x, nb[k], r_ij.x * 0.5);
    for (int j = 0; j < nt; ++j) {
      if (k == 0) {
        tvx[j] = t->ct[j] * (r_ij.x * 0.5);
        tvy[j] = t->ct[j] * (r_ij.y * 0.5);
      } else {
        tvx[j] += t->ct[j] * (r_ij.x * 0.5);
        tvy[j] += t->ct[j] * (r_ij.y * 0.5);
      }
      tvy[j] += t->nb[k][j] * (r_ij.y * 0.5);
      tvx[j] += t->nb[k][j] * (r_ij.x * 0.5);
    }
  }
  mm[0] += vol;
  mm[3] += vol;
  const double det = mm[0] * mm[3] - mm[1] * mm[2];
  if (fabs(det) < 1e-10 * vol * vol) {
    set_err(err, RG_ERR_SINGULAR_MATRIX, 2, i, det);
    return RG_ERR_SINGULAR_MATRIX;
  }
  const double det_inv = 1.0 / det;
  const double mi0 = mm[3] * det_inv, mi1 = -mm[1] * det_inv, mi2 = -mm[2] * det_inv, mi3 = mm[0] * det_inv;
  res->x = ccscale(vc.x, mi0);
  res->y = ccscale(vc.y, mi3);
  addmult(&res->x, vc.y, mi1);
  addmult(&res->y, vc.x, mi2);
  for (int j = 0; j < nt; ++j) {
    t->sx[j] = tvx[j] * mi0;
    t->sy[j] = tvy[j] * mi3;
    t->sx[j] += tvy[j] * mi1;
    t->sy[j] += tvx[j] * mi2;
  }
  return 0;
}

/* :401-422 GetBoundarySlope */
static void boundary_slope(cc cell, v2 cell_cm, int n, const cc* nb, const v2* nb_cm, slope* res, trcell* t) {
  cc phisy = {0, 0, 0, 0}, phisx = {0, 0, 0, 0};
  double tpy[RG_MAX_TRACERS] = {0}, tpx[RG_MAX_TRACERS] = {0};
  const int nt = t ? t->nt : 0;
  double sxsy = 0, sy2 = 0, sx2 = 0;
  for (int k = 0; k < n; ++k) {
    phisy = ccadd(phisy, ccscale(ccsub(nb[k], cell), nb_cm[k].y - cell_cm.y));
    phisx = ccadd(phisx, ccscale(ccsub(nb[k], cell), nb_cm[k].x - cell_cm.x));
    for (int j = 0; j < nt; ++j) {
      tpy[j] = tpy[j] + (t->nb[k][j] - t->ct[j]) * (nb_cm[k].y - cell_cm.y);
      tpx[j] = tpx[j] + (t->nb[k][j] - t->ct[j]) * (nb_cm[k].x - cell_cm.x);
    }
    sxsy += (nb_cm[k].y - cell_cm.y) * (nb_cm[k].x - cell_cm.x);
    sx2 += (nb_cm[k].x - cell_cm.x) * (nb_cm[k].x - cell_cm.x);
    sy2 += (nb_cm[k].y - cell_cm.y) * (nb_cm[k].y - cell_cm.y);
  }
  const double den = sxsy * sxsy - sx2 * sy2;
  const cc ax = ccsub(ccscale(phisy, sxsy), ccscale(phisx, sy2));
  const cc ay = ccsub(ccscale(phisx, sxsy), ccscale(phisy, sx2));
  res->x.d = ax.d / den; res->x.p = ax.p / den; res->x.vx = ax.vx / den; res->x.vy = ax.vy / den;
  res->y.d = ay.d / den; res->y.p = ay.p / den; res->y.vx = ay.vx / den; res->y.vy = ay.vy / den;
  for (int j = 0; j < nt; ++j) {
    t->sx[j] = (tpy[j] * sxsy - tpx[j] * sy2) / den;
    t->sy[j] = (tpx[j] * sxsy - tpy[j] * sx2) / den;
  }
}

/* :136-148 PressureRatio, :150-157 is_shock */
static int is_shock(slope naive, double cell_width, double shockratio, cc cell, int n, const cc* nb,
                    double pressure_ratio, double cs) {
  const int cond1 = (naive.x.vx + naive.y.vy) * cell_width < (-shockratio) * cs;
  double res = 1;
  const double p = cell.p;
  for (int k = 0; k < n; ++k) {
    if (p > nb[k].p)
      res = smin(res, nb[k].p / p);
    else
      res = smin(res, p / nb[k].p);
  }
  const int cond2 = res < pressure_ratio;
  return cond1 || cond2;
}

/* one ComputationalCell component of :232-267 (ordinary limiter).  velocity
 * thresholds use |1e-9*v|, density/pressure thresholds 1e-9*q (no abs). */
static void limit_comp(double dphi, double cv, double cellv, double maxd, double mind, int use_abs,
                       double* psi) {
  if (fabs(dphi) > 0.05 * smax(fabs(maxd), fabs(mind)) || cv * cellv < 0) {
    const double thr = use_abs ? fabs(1e-9 * cellv) : 1e-9 * cellv;
    const double nthr = use_abs ? -fabs(1e-9 * cellv) : -1e-9 * cellv;
    if (dphi > thr)
      *psi = smin(*psi, maxd / dphi);
    else if (dphi < nthr)
      *psi = smin(*psi, mind / dphi);
  }
}

/* :174-300 slope_limit */
static void slope_limit(const rg_mesh_view* m, cc cell, v2 cm, int n, const cc* nb, const int* edges,
                        const int* skip, slope* s, trcell* t) {
  const int nt = t ? t->nt : 0;
  cc cmax = cell, cmin = cell;
  double tmax[RG_MAX_TRACERS], tmin[RG_MAX_TRACERS], tpsi[RG_MAX_TRACERS];
  for (int j = 0; j < nt; ++j) {
    tmax[j] = tmin[j] = t->ct[j];
    tpsi[j] = 1;
  }
  for (int k = 0; k < n; ++k) {
    const int e = edges[k];
    if (skip[k]) continue; /* :192-193 neighbours with the skip_key sticker */
    if (orig(m, fc0(m, e)) == orig(m, fc1(m, e))) continue;
    for (int j = 0; j < nt; ++j) {
      tmax[j] = smax(tmax[j], t->nb[k][j]);
      tmin[j] = smin(tmin[j], t->nb[k][j]);
    }
    cmax.d = smax(cmax.d, nb[k].d);
    cmax.p = smax(cmax.p, nb[k].p);
    cmax.vx = smax(cmax.vx, nb[k].vx);
    cmax.vy = smax(cmax.vy, nb[k].vy);
    cmin.d = smin(cmin.d, nb[k].d);
    cmin.p = smin(cmin.p, nb[k].p);
    cmin.vx = smin(cmin.vx, nb[k].vx);
    cmin.vy = smin(cmin.vy, nb[k].vy);
  }
  const cc maxdiff = ccsub(cmax, cell), mindiff = ccsub(cmin, cell);
  double psi[4] = {1, 1, 1, 1};
  for (int k = 0; k < n; ++k) {
    cc cv = cell;
    const v2 target = centroid(m, edges[k]);
    interp2(&cv, *s, target, cm);
    const cc dphi = ccsub(cv, cell);
    limit_comp(dphi.d, cv.d, cell.d, maxdiff.d, mindiff.d, 0, &psi[0]);
    limit_comp(dphi.p, cv.p, cell.p, maxdiff.p, mindiff.p, 0, &psi[1]);
    limit_comp(dphi.vx, cv.vx, cell.vx, maxdiff.vx, mindiff.vx, 1, &psi[2]);
    limit_comp(dphi.vy, cv.vy, cell.vy, maxdiff.vy, mindiff.vy, 1, &psi[3]);
    /* :268-283 tracers: the velocity form, |1e-9*tracer| dead band */
    for (int j = 0; j < nt; ++j) {
      double cvt = t->ct[j];
      cvt += t->sx[j] * (target.x - cm.x);
      cvt += t->sy[j] * (target.y - cm.y);
      limit_comp(cvt - t->ct[j], cvt, t->ct[j], tmax[j] - t->ct[j], tmin[j] - t->ct[j], 1, &tpsi[j]);
    }
  }
  s->x.d *= psi[0]; s->y.d *= psi[0];
  s->x.p *= psi[1]; s->y.p *= psi[1];
  s->x.vx *= psi[2]; s->y.vx *= psi[2];
  s->x.vy *= psi[3]; s->y.vy *= psi[3];
  for (int j = 0; j < nt; ++j) {
    t->sx[j] *= tpsi[j];
    t->sy[j] *= tpsi[j];
  }
}

/* one component of :343-366 (shocked limiter); the threshold is 1e-9*q
 * without abs for every component, as in the reference (:346,352,358,364). */
static void shocked_comp(double dphi, double cv, double cellv, double maxd, double mind, double nbv,
                         double theta, double* psi) {
  if (fabs(dphi) > 0.1 * smax(fabs(maxd), fabs(mind)) || cv * cellv < 0) {
    if (fabs(dphi) > 1e-9 * cellv) *psi = smin(*psi, smax(theta * (nbv - cellv) / dphi, 0.0));
  }
}

/* :302-399 shocked_slope_limit */
static void shocked_slope_limit(const rg_mesh_view* m, cc cell, v2 cm, int n, const cc* nb,
                                const int* edges, const int* skip, double theta, slope* s, trcell* t) {
  const int nt = t ? t->nt : 0;
  cc cmax = cell, cmin = cell;
  double tmax[RG_MAX_TRACERS], tmin[RG_MAX_TRACERS], tpsi[RG_MAX_TRACERS];
  for (int j = 0; j < nt; ++j) {
    tmax[j] = tmin[j] = t->ct[j];
    tpsi[j] = 1;
  }
  for (int k = 0; k < n; ++k) {
    if (skip[k]) continue; /* :314-315 */
    for (int j = 0; j < nt; ++j) {
      tmax[j] = smax(tmax[j], t->nb[k][j]);
      tmin[j] = smin(tmin[j], t->nb[k][j]);
    }
    cmax.d = smax(cmax.d, nb[k].d);
    cmax.p = smax(cmax.p, nb[k].p);
    cmax.vx = smax(cmax.vx, nb[k].vx);
    cmax.vy = smax(cmax.vy, nb[k].vy);
    cmin.d = smin(cmin.d, nb[k].d);
    cmin.p = smin(cmin.p, nb[k].p);
    cmin.vx = smin(cmin.vx, nb[k].vx);
    cmin.vy = smin(cmin.vy, nb[k].vy);
  }
  const cc maxdiff = ccsub(cmax, cell), mindiff = ccsub(cmin, cell);
  double psi[4] = {1, 1, 1, 1};
  for (int k = 0; k < n; ++k) {
    if (skip[k]) continue; /* :339-340 */
    cc cv = cell;
    const v2 target = centroid(m, edges[k]);
    interp2(&cv, *s, target, cm);
    const cc dphi = ccsub(cv, cell);
    shocked_comp(dphi.d, cv.d, cell.d, maxdiff.d, mindiff.d, nb[k].d, theta, &psi[0]);
    shocked_comp(dphi.p, cv.p, cell.p, maxdiff.p, mindiff.p, nb[k].p, theta, &psi[1]);
    shocked_comp(dphi.vx, cv.vx, cell.vx, maxdiff.vx, mindiff.vx, nb[k].vx, theta, &psi[2]);
    shocked_comp(dphi.vy, cv.vy, cell.vy, maxdiff.vy, mindiff.vy, nb[k].vy, theta, &psi[3]);
    /* :367-385 tracers: threshold |1e-9*tracer| */
    for (int j = 0; j < nt; ++j) {
      const double ctj = t->ct[j];
      double cvt = ctj;
      cvt += t->sx[j] * (target.x - cm.x);
      cvt += t->sy[j] * (target.y - cm.y);
      const double dphi_t = cvt - ctj, maxd = tmax[j] - ctj, mind = tmin[j] - ctj;
      if (fabs(dphi_t) > 0.1 * smax(fabs(maxd), fabs(mind)) || cvt * ctj < 0) {
        if (fabs(dphi_t) > fabs(1e-9 * ctj))
          tpsi[j] = smin(tpsi[j], smax(theta * (t->nb[k][j] - ctj) / dphi_t, 0.0));
      }
    }
  }
  s->x.d *= psi[0]; s->y.d *= psi[0];
  s->x.p *= psi[1]; s->y.p *= psi[1];
  s->x.vx *= psi[2]; s->y.vx *= psi[2];
  s->x.vy *= psi[3]; s->y.vy *= psi[3];
  for (int j = 0; j < nt; ++j) {
    t->sx[j] *= tpsi[j];
    t->sy[j] *= tpsi[j];
  }
}

static void put_cc(double* o, cc c) { o[0] = c.d; o[1] = c.p; o[2] = c.vx; o[3] = c.vy; }
static cc get_cc(const double* o) { cc c = {o[0], o[1], o[2], o[3]}; return c; }

/* The cell whose tracers and stickers point p carries: p itself, or the cell
 * a ghost copies (PeriodicGhostGenerator.cpp:3-17: the source;
 * RigidWallGenerator.cpp:17-37: the real side of the ghost's face); -1 for
 * a ghost on no face. */
static int copied_cell(const rg_mesh_view* m, int p, int ghost_kind) {
  const int N = m->n_cells;
  if (p < N) return p;
  const int g = p - N;
  if (ghost_kind == RG_GHOST_PERIODIC) return m->ghost_source[g];
  const int e = m->ghost_face[g];
  if (e < 0) return -1;
  return fc0(m, e) >= N ? fc1(m, e) : fc0(m, e);
}

static uint32_t stickers_of(const ro_tracers* t, int c) {
  return t && t->stickers && c >= 0 ? t->stickers[c] : 0u;
}

/* :536-635 LinearGaussImproved::operator() (serial build), with :425-494 calc_slope */
int ro_lgi_tr(const rg_mesh_view* m, const double* cells, const double* tr, double g, const ro_lgi_params* lp,
              const ro_tracers* t, double* slopes, double* interp, double* tslopes, double* tinterp,
              ro_error* err) {
  const int N = m->n_cells;
  const int nt = t ? t->n : 0;
  cc* gs = (cc*)calloc((size_t)(m->n_ghosts > 0 ? m->n_ghosts : 1), sizeof(cc));
  slope* sl = (slope*)calloc((size_t)N, sizeof(slope));
  double* tsl = (double*)calloc((size_t)N * 2 * (nt > 0 ? nt : 1), sizeof(double));
  trcell* tc = nt > 0 ? (trcell*)calloc(1, sizeof(trcell)) : NULL;
  int st = 0;
  ghost_states(m, cells, lp->ghost_kind, gs);
  for (int i = 0; i < N && !st; ++i) {
    const int b = m->cell_face_offset[i], n = m->cell_face_offset[i + 1] - b;
    const int* edges = m->cell_faces + b;
    cc nb[RO_MAX_NB];
    v2 nb_pt[RO_MAX_NB], nb_cm[RO_MAX_NB];
    int skip[RO_MAX_NB];
    if (n > RO_MAX_NB) {
      set_err(err, RG_ERR_TOO_MANY_NEIGHBORS, 2, i, n);
      st = RG_ERR_TOO_MANY_NEIGHBORS;
      break;
    }
    if (tc) {
      tc->nt = nt;
      for (int j = 0; j < nt; ++j) tc->ct[j] = tr[(size_t)i * nt + j];
    }
    int bslope = 0;
    for (int k = 0; k < n; ++k) {
      const int e = edges[k];
      const int other = fc0(m, e) == i ? fc1(m, e) : fc0(m, e);
      nb[k] = any_state(m, cells, gs, other);
      nb_pt[k] = point(m, other);
      nb_cm[k] = cmof(m, other);
      if (orig(m, fc0(m, e)) == orig(m, fc1(m, e))) bslope = 1;
      const int src = copied_cell(m, other, lp->ghost_kind);
      skip[k] = t && t->skip_mask && (stickers_of(t, src) & t->skip_mask) != 0;
      for (int j = 0; j < nt; ++j) tc->nb[k][j] = src >= 0 ? tr[(size_t)src * nt + j] : 0.0;
    }
    const cc cell = cell_at(cells, i);
    slope s;
    if (bslope)
      boundary_slope(cell, cmof(m, i), n, nb, nb_cm, &s, tc);
    else {
      st = naive_slope(m, i, cell, point(m, i), cmof(m, i), m->volume[i], edges, n, nb, nb_pt, nb_cm, &s, tc, err);
      if (st) break;
    }
    /* :470-479 tracers outside calc_tracers get zero slopes */
    for (int j = 0; j < nt; ++j)
      if (!((t->limited >> j) & 1u)) tc->sx[j] = tc->sy[j] = 0;
    if (lp->slf) {
      if (!is_shock(s, width(m, i), lp->delta_v, cell, n, nb, lp->delta_p, dp2c(g, cell.d, cell.p)))
        slope_limit(m, cell, cmof(m, i), n, nb, edges, skip, &s, tc);
      else
        shocked_slope_limit(m, cell, cmof(m, i), n, nb, edges, skip, lp->theta, &s, tc);
    }
    sl[i] = s;
    if (slopes) {
      put_cc(slopes + 8 * i, s.x);
      put_cc(slopes + 8 * i + 4, s.y);
    }
    for (int j = 0; j < nt; ++j) {
      tsl[(size_t)i * 2 * nt + j] = tc->sx[j];
      tsl[(size_t)i * 2 * nt + nt + j] = tc->sy[j];
    }
    /* :570-590 interpolation of the real side of each edge */
    for (int k = 0; k < n; ++k) {
      const int e = edges[k];
      cc r = cell;
      const v2 target = centroid(m, e), cm = cmof(m, i);
      interp2(&r, s, target, cm);
      const int side = fc0(m, e) == i ? 0 : 1;
      put_cc(interp + 8 * e + 4 * side, r);
      for (int j = 0; j < nt; ++j) {
        double rt = tc->ct[j];
        rt += tc->sx[j] * (target.x - cm.x);
        rt += tc->sy[j] * (target.y - cm.y);
        if (tinterp) tinterp[(size_t)e * 2 * nt + (size_t)side * nt + j] = rt;
      }
    }
  }
  if (!st) {
    /* :596-634 ghost side of boundary edges: ghost state + ghost gradient */
    for (int e = 0; e < m->n_faces; ++e) {
      const int a = fc0(m, e), b = fc1(m, e);
      int side, gp;
      if (a >= N) { side = 0; gp = a; }
      else if (b >= N) { side = 1; gp = b; }
      else continue;
      cc r = gs[gp - N];
      slope gg;
      const int periodic = lp->ghost_kind == RG_GHOST_PERIODIC;
      if (periodic)
        gg = sl[orig(m, gp)];
      else
        memset(&gg, 0, sizeof gg);
      const v2 target = centroid(m, e), cm = cmof(m, gp);
      interp2(&r, gg, target, cm);
      put_cc(interp + 8 * e + 4 * side, r);
      /* tracers: the copied cell's values; periodic ghosts take the source's
       * gradient, rigid walls a zero one (RigidWallGenerator.cpp:39-54) */
      const int src = copied_cell(m, gp, lp->ghost_kind);
      for (int j = 0; j < nt; ++j) {
        double rt = src >= 0 ? tr[(size_t)src * nt + j] : 0.0;
        const double gx = periodic ? tsl[(size_t)orig(m, gp) * 2 * nt + j] : 0.0;
        const double gy = periodic ? tsl[(size_t)orig(m, gp) * 2 * nt + nt + j] : 0.0;
        rt += gx * (target.x - cm.x);
        rt += gy * (target.y - cm.y);
        if (tinterp) tinterp[(size_t)e * 2 * nt + (size_t)side * nt + j] = rt;
      }
    }
  }
  if (tslopes && nt > 0) memcpy(tslopes, tsl, sizeof(double) * (size_t)N * 2 * nt);
  free(gs);
  free(sl);
  free(tsl);
  free(tc);
  return st;
}

int ro_lgi(const rg_mesh_view* m, const double* cells, double g, const ro_lgi_params* lp,
           double* slopes, double* interp, ro_error* err) {
  return ro_lgi_tr(m, cells, NULL, g, lp, NULL, slopes, interp, NULL, NULL, err);
}

/* modular_flux_calculator.cpp:12-22 calc_parallel_normal and
 * simple_flux_calculator.cpp:27-31 remove_parallel_component */
static v2 remove_parallel(v2 v, v2 p) { return vsub(v, vdiv(vscale(p, dot(v, p)), dot(p, p))); }

/* modular_flux_calculator.cpp:39-71, tracer fluxes :24-35
 * (convert_conserved_to_extensive: Mass * the first side's interpolated
 * tracer when Mass > 0, else the second side's) */
int ro_modular_flux_tr(const rg_mesh_view* m, const double* cells, const double* tr, const double* ev, double g,
                       const ro_lgi_params* lp, const ro_tracers* t, double* fluxes, double* tfluxes,
                       ro_error* err) {
  const int N = m->n_cells;
  const int nt = t ? t->n : 0;
  const size_t E = (size_t)(m->n_faces > 0 ? m->n_faces : 1);
  double* ip = (double*)malloc(sizeof(double) * 8 * E);
  double* tip = nt > 0 ? (double*)malloc(sizeof(double) * 2 * nt * E) : NULL;
  int st = ro_lgi_tr(m, cells, tr, g, lp, t, NULL, ip, NULL, tip, err);
  for (int e = 0; e < m->n_faces && !st; ++e) {
    const int a = fc0(m, e), b = fc1(m, e);
    const v2 p = parallel(m, e);
    v2 n;
    if (a >= 0 && a < N)
      n = remove_parallel(vsub(vert0(m, e), point(m, a)), p);
    else
      n = remove_parallel(vsub(point(m, b), vert0(m, e)), p);
    const v2 w = {ev[2 * e], ev[2 * e + 1]};
    const double speed = dot(n, w) / vabs(n);
    const prim pl = to_prim(g, get_cc(ip + 8 * e)), pr = to_prim(g, get_cc(ip + 8 * e + 4));
    cons c;
    st = rotate_solve_rotate_back(pl, pr, speed, n, p, &c, e, err);
    if (st) break;
    put_flux(fluxes + 4 * e, c);
    for (int j = 0; j < nt; ++j)
      tfluxes[(size_t)e * nt + j] = c.m * (c.m > 0 ? tip[(size_t)e * 2 * nt + j] : tip[(size_t)e * 2 * nt + nt + j]);
  }
  free(ip);
  free(tip);
  return st;
}

int ro_modular_flux(const rg_mesh_view* m, const double* cells, const double* ev, double g,
                    const ro_lgi_params* lp, double* fluxes, ro_error* err) {
  return ro_modular_flux_tr(m, cells, NULL, ev, g, lp, NULL, fluxes, NULL, err);
}

/* simple_flux_calculator.cpp:193-213 calc_tracer_flux: Mass times the
 * upwind point's tracer, 0 when the upwind point is a self-mirror ghost (or
 * Mass is 0).  A non-mirror ghost (periodic) reads the tracer of its source
 * cell, as the hydro state does. */
int ro_simple_flux_tr(const rg_mesh_view* m, const double* cells, const double* tr, const double* ev, double g,
                      const ro_tracers* t, double* fluxes, double* tfluxes, ro_error* err) {
  const int st = ro_simple_flux(m, cells, ev, g, fluxes, err);
  const int nt = t ? t->n : 0;
  if (st || nt == 0) return st;
  const int N = m->n_cells;
  for (int e = 0; e < m->n_faces; ++e) {
    const int a = fc0(m, e), b = fc1(m, e);
    const double mass = fluxes[4 * e];
    const int mirror = orig(m, a) == orig(m, b);
    int up = -1;
    if (mass > 0 && a >= 0 && (a < N || !mirror))
      up = a;
    else if (mass < 0 && b >= 0 && (b < N || !mirror))
      up = b;
    for (int j = 0; j < nt; ++j)
      tfluxes[(size_t)e * nt + j] = up >= 0 ? mass * tr[(size_t)orig(m, up) * nt + j] : 0.0;
  }
  return 0;
}

/* simple_extensive_updater.cpp:11-35 */
int ro_extensive_update(const rg_mesh_view* m, const double* fluxes, double dt, double* ext,
                        ro_error* err) {
  (void)err;
  const int N = m->n_cells;
  for (int e = 0; e < m->n_faces; ++e) {
    const double s = dt * edge_area(m, e);
    const double dm = fluxes[4 * e] * s, de = fluxes[4 * e + 1] * s;
    const double dx = fluxes[4 * e + 2] * s, dy = fluxes[4 * e + 3] * s;
    const int a = fc0(m, e), b = fc1(m, e);
    if (a >= 0 && a < N) {
      ext[4 * a] -= dm;
      ext[4 * a + 1] -= de;
      ext[4 * a + 2] -= dx;
      ext[4 * a + 3] -= dy;
    }
    if (b >= 0 && b < N) {
      ext[4 * b] += dm;
      ext[4 * b + 1] += de;
      ext[4 * b + 2] += dx;
      ext[4 * b + 3] += dy;
    }
  }
  return 0;
}

/* simple_cell_updater.cpp:22-59 regular_update, :85-106 operator() */
int ro_cell_update(const rg_mesh_view* m, const double* ext, double g, double* cells_out,
                   ro_error* err) {
  for (int i = 0; i < m->n_cells; ++i) {
    const double mass = ext[4 * i], en = ext[4 * i + 1], px = ext[4 * i + 2], py = ext[4 * i + 3];
    const double volume = m->cd_volume[i];
    const double d = mass / volume;
    if (d < 0) {
      set_err(err, RG_ERR_NEGATIVE_DENSITY, 5, i, d);
      return RG_ERR_NEGATIVE_DENSITY;
    }
    const double vx = px / mass, vy = py / mass;
    const double energy = en / mass - 0.5 * (vx * vx + vy * vy);
    if (energy < 0) {
      set_err(err, RG_ERR_NEGATIVE_ENERGY, 5, i, energy);
      return RG_ERR_NEGATIVE_ENERGY;
    }
    cells_out[4 * i] = d;
    cells_out[4 * i + 1] = (g - 1) * energy * d;
    cells_out[4 * i + 2] = vx;
    cells_out[4 * i + 3] = vy;
  }
  return 0;
}

/* hdsim2d.cpp:41-67 init_extensives (volume = pg.calcVolume = cd_volume) */
int ro_init_extensives(const rg_mesh_view* m, const double* cells, double g, double* ext) {
  for (int i = 0; i < m->n_cells; ++i) {
    const double d = cells[4 * i], p = cells[4 * i + 1], vx = cells[4 * i + 2], vy = cells[4 * i + 3];
    const double mass = m->cd_volume[i] * d;
    ext[4 * i] = mass;
    ext[4 * i + 1] = dp2e(g, d, p) * mass + 0.5 * mass * (vx * vx + vy * vy);
    ext[4 * i + 2] = vx * mass;
    ext[4 * i + 3] = vy * mass;
  }
  return 0;
}

/* simple_extensive_updater.cpp:11-35 for the extensive tracers: delta =
 * flux * (dt*area), subtracted from the first cell, added to the second */
void ro_extensive_update_tr(const rg_mesh_view* m, const double* tfluxes, int nt, double dt, double* tr_ext) {
  const int N = m->n_cells;
  for (int e = 0; e < m->n_faces; ++e) {
    const double s = dt * edge_area(m, e);
    const int a = fc0(m, e), b = fc1(m, e);
    for (int j = 0; j < nt; ++j) {
      const double d = tfluxes[(size_t)e * nt + j] * s;
      if (a >= 0 && a < N) tr_ext[(size_t)a * nt + j] -= d;
      if (b >= 0 && b < N) tr_ext[(size_t)b * nt + j] += d;
    }
  }
}

/* simple_cell_updater.cpp:61-83 update_single with the sequence
 * {(HasSticker(frozen), SkipUpdate())} (:107-140: the old cell, tracers and
 * stickers included), else :22-59 regular_update: tracers = extensive
 * tracers / mass, the "Entropy" tracer = IdealGas::dp2s (ideal_gas.cpp:52-55,
 * p*pow(d,-gamma)) with its extensive set to s*mass. */
int ro_cell_update_tr(const rg_mesh_view* m, const double* ext, double* tr_ext, const double* old_cells,
                      const double* old_tr, double g, const ro_tracers* t, double* cells_out, double* tr_out,
                      ro_error* err) {
  const int nt = t ? t->n : 0;
  for (int i = 0; i < m->n_cells; ++i) {
    if (t && t->frozen_mask && t->stickers && (t->stickers[i] & t->frozen_mask)) {
      memcpy(cells_out + 4 * i, old_cells + 4 * i, 4 * sizeof(double));
      for (int j = 0; j < nt; ++j) tr_out[(size_t)i * nt + j] = old_tr[(size_t)i * nt + j];
      continue;
    }
    const double mass = ext[4 * i], en = ext[4 * i + 1], px = ext[4 * i + 2], py = ext[4 * i + 3];
    const double d = mass / m->cd_volume[i];
    if (d < 0) {
      set_err(err, RG_ERR_NEGATIVE_DENSITY, 5, i, d);
      return RG_ERR_NEGATIVE_DENSITY;
    }
    const double vx = px / mass, vy = py / mass;
    const double energy = en / mass - 0.5 * (vx * vx + vy * vy);
    for (int j = 0; j < nt; ++j) tr_out[(size_t)i * nt + j] = tr_ext[(size_t)i * nt + j] / mass;
    if (energy < 0) {
      set_err(err, RG_ERR_NEGATIVE_ENERGY, 5, i, energy);
      return RG_ERR_NEGATIVE_ENERGY;
    }
    const double pres = (g - 1) * energy * d;
    cells_out[4 * i] = d;
    cells_out[4 * i + 1] = pres;
    cells_out[4 * i + 2] = vx;
    cells_out[4 * i + 3] = vy;
    if (t && t->entropy >= 0 && t->entropy < nt) {
      const double sv = pres * pow(d, -g);
      tr_out[(size_t)i * nt + t->entropy] = sv;
      tr_ext[(size_t)i * nt + t->entropy] = sv * mass;
    }
  }
  return 0;
}

/* hdsim2d.cpp:56-63 init_extensives: tracer * mass */
void ro_init_extensives_tr(const rg_mesh_view* m, const double* cells, const double* tr, int nt, double* tr_ext) {
  for (int i = 0; i < m->n_cells; ++i) {
    const double mass = m->cd_volume[i] * cells[4 * i];
    for (int j = 0; j < nt; ++j) tr_ext[(size_t)i * nt + j] = tr[(size_t)i * nt + j] * mass;
  }
}

/* simple_cfl.cpp:28-47 TimeStepCalculator, :58-71 operator(), lazy_list.hpp:185-191 lazy_min */
int ro_cfl(const rg_mesh_view* m, const double* cells, const double* ev, double g, double cfl,
           double* dt, ro_error* err) {
  (void)err;
  double best = 0;
  for (int i = 0; i < m->n_cells; ++i) {
    double res = 0;
    const double radius = width(m, i);
    const double c = dp2c(g, cells[4 * i], cells[4 * i + 1]);
    const v2 v = {cells[4 * i + 2], cells[4 * i + 3]};
    for (int k = m->cell_face_offset[i]; k < m->cell_face_offset[i + 1]; ++k) {
      const int e = m->cell_faces[k];
      const v2 ve = {ev[2 * e], ev[2 * e + 1]};
      res = fmax(res, (c + vabs(vsub(v, ve))) / radius);
    }
    const double x = 1.0 / res;
    best = i == 0 ? x : smin(best, x);
  }
  *dt = cfl * best;
  return 0;
}

int ro_step(const rg_mesh_view* m, double* cells, double* ext, const double* ev, double g,
            double cfl, int order, const ro_lgi_params* lp, double* dt_out, ro_error* err) {
  double dt;
  int st = ro_cfl(m, cells, ev, g, cfl, &dt, err);
  if (st) return st;
  double* fl = (double*)malloc(sizeof(double) * 4 * (size_t)(m->n_faces > 0 ? m->n_faces : 1));
  st = order == 1 ? ro_simple_flux(m, cells, ev, g, fl, err) : ro_modular_flux(m, cells, ev, g, lp, fl, err);
  if (!st) st = ro_extensive_update(m, fl, dt, ext, err);
  if (!st) st = ro_cell_update(m, ext, g, cells, err);
  free(fl);
  if (dt_out) *dt_out = dt;
  return st;
}

int ro_step_tr(const rg_mesh_view* m, double* cells, double* ext, double* tr, double* tr_ext, const double* ev,
               double g, double cfl, int order, const ro_lgi_params* lp, const ro_tracers* t, double* dt_out,
               ro_error* err) {
  double dt;
  int st = ro_cfl(m, cells, ev, g, cfl, &dt, err);
  if (st) return st;
  const int nt = t ? t->n : 0;
  const size_t E = (size_t)(m->n_faces > 0 ? m->n_faces : 1), N = (size_t)m->n_cells;
  double* fl = (double*)malloc(sizeof(double) * 4 * E);
  double* tfl = (double*)malloc(sizeof(double) * E * (nt > 0 ? nt : 1));
  double* old_cells = (double*)malloc(sizeof(double) * 4 * N);
  double* old_tr = (double*)malloc(sizeof(double) * N * (nt > 0 ? nt : 1));
  memcpy(old_cells, cells, sizeof(double) * 4 * N);
  if (nt > 0) memcpy(old_tr, tr, sizeof(double) * N * nt);
  st = order == 1 ? ro_simple_flux_tr(m, cells, tr, ev, g, t, fl, tfl, err)
                  : ro_modular_flux_tr(m, cells, tr, ev, g, lp, t, fl, tfl, err);
  if (!st) st = ro_extensive_update(m, fl, dt, ext, err);
  if (!st) ro_extensive_update_tr(m, tfl, nt, dt, tr_ext);
  if (!st) st = ro_cell_update_tr(m, ext, tr_ext, old_cells, old_tr, g, t, cells, tr, err);
  free(fl);
  free(tfl);
  free(old_cells);
  free(old_tr);
  if (dt_out) *dt_out = dt;
  return st;
}

int ro_step_heun_tr(const rg_mesh_view* m, double* cells, double* ext, double* tr, double* tr_ext,
                    const double* ev, double g, double cfl, int order, const ro_lgi_params* lp, const ro_tracers* t,
                    double* dt_out, ro_error* err) {
  double dt;
  int st = ro_cfl(m, cells, ev, g, cfl, &dt, err);
  if (st) return st;
  const int nt = t ? t->n : 0;
  const size_t E = (size_t)(m->n_faces > 0 ? m->n_faces : 1), N = (size_t)m->n_cells;
  const size_t ntr = N * (size_t)(nt > 0 ? nt : 1);
  double* fl = (double*)malloc(sizeof(double) * 4 * E);
  double* tfl = (double*)malloc(sizeof(double) * E * (nt > 0 ? nt : 1));
  double* mid = (double*)malloc(sizeof(double) * 4 * N);
  double* mid_cells = (double*)malloc(sizeof(double) * 4 * N);
  double* mid_tr = (double*)malloc(sizeof(double) * ntr);
  double* mid_tr_ext = (double*)malloc(sizeof(double) * ntr);
  memcpy(mid, ext, sizeof(double) * 4 * N);
  if (nt > 0) memcpy(mid_tr_ext, tr_ext, sizeof(double) * N * nt);
  /* first half: fluxes of the step's cells, mid = ext + dt*area*F1, mid cells */
  st = order == 1 ? ro_simple_flux_tr(m, cells, tr, ev, g, t, fl, tfl, err)
                  : ro_modular_flux_tr(m, cells, tr, ev, g, lp, t, fl, tfl, err);
  if (!st) st = ro_extensive_update(m, fl, dt, mid, err);
  if (!st) ro_extensive_update_tr(m, tfl, nt, dt, mid_tr_ext);
  if (!st) st = ro_cell_update_tr(m, mid, mid_tr_ext, cells, tr, g, t, mid_cells, mid_tr, err);
  /* second half: fluxes of the mid cells, mid += dt*area*F2 */
  if (!st)
    st = order == 1 ? ro_simple_flux_tr(m, mid_cells, mid_tr, ev, g, t, fl, tfl, err)
                    : ro_modular_flux_tr(m, mid_cells, mid_tr, ev, g, lp, t, fl, tfl, err);
  if (!st) st = ro_extensive_update(m, fl, dt, mid, err);
  if (!st) ro_extensive_update_tr(m, tfl, nt, dt, mid_tr_ext);
  if (!st) {
    /* average_extensive (hdsim2d.cpp:311-320), then the cells from it */
    for (size_t k = 0; k < 4 * N; ++k) ext[k] = 0.5 * (mid[k] + ext[k]);
    for (size_t k = 0; k < N * (size_t)nt; ++k) tr_ext[k] = 0.5 * (mid_tr_ext[k] + tr_ext[k]);
    double* old_cells = (double*)malloc(sizeof(double) * 4 * N);
    double* old_tr = (double*)malloc(sizeof(double) * ntr);
    memcpy(old_cells, cells, sizeof(double) * 4 * N);
    if (nt > 0) memcpy(old_tr, tr, sizeof(double) * N * nt);
    st = ro_cell_update_tr(m, ext, tr_ext, old_cells, old_tr, g, t, cells, tr, err);
    free(old_cells);
    free(old_tr);
  }
  free(fl);
  free(tfl);
  free(mid);
  free(mid_cells);
  free(mid_tr);
  free(mid_tr_ext);
  if (dt_out) *dt_out = dt;
  return st;
}

/* hdsim2d.cpp:323-449 TimeAdvance2Heun with ZeroForce (which adds dt*0) and a
 * mesh that does not move: dt, F1 on the cells, mid = ext + dt*area*F1,
 * mid cells, F2 on the mid cells, mid += dt*area*F2, ext = 0.5*(mid + ext)
 * (average_extensive, hdsim2d.cpp:311-320), cells from ext. */
int ro_step_heun(const rg_mesh_view* m, double* cells, double* ext, const double* ev, double g,
                 double cfl, int order, const ro_lgi_params* lp, double* dt_out, ro_error* err) {
  double dt;
  int st = ro_cfl(m, cells, ev, g, cfl, &dt, err);
  if (st) return st;
  const size_t n4 = 4 * (size_t)m->n_cells;
  double* fl = (double*)malloc(sizeof(double) * 4 * (size_t)(m->n_faces > 0 ? m->n_faces : 1));
  double* mid = (double*)malloc(sizeof(double) * n4);
  double* mid_cells = (double*)malloc(sizeof(double) * n4);
  memcpy(mid, ext, sizeof(double) * n4);
  st = order == 1 ? ro_simple_flux(m, cells, ev, g, fl, err) : ro_modular_flux(m, cells, ev, g, lp, fl, err);
  if (!st) st = ro_extensive_update(m, fl, dt, mid, err);
  if (!st) st = ro_cell_update(m, mid, g, mid_cells, err);
  if (!st)
    st = order == 1 ? ro_simple_flux(m, mid_cells, ev, g, fl, err)
                    : ro_modular_flux(m, mid_cells, ev, g, lp, fl, err);
  if (!st) st = ro_extensive_update(m, fl, dt, mid, err);
  if (!st) {
    for (size_t k = 0; k < n4; ++k) ext[k] = 0.5 * (mid[k] + ext[k]);
    st = ro_cell_update(m, ext, g, cells, err);
  }
  free(fl);
  free(mid);
  free(mid_cells);
  if (dt_out) *dt_out = dt;
  return st;
}

/* ========================================================================
 * Geometry and point motion (tessellation, CacheData, PointMotion,
 * EdgeVelocityCalculator)
 * ======================================================================== */

/* geometry.cpp:138-141 zcross, :100-104 ScalarProd: 0.5*|p1 . zcross(p2)| */
static double half_cross(v2 p1, v2 p2) {
  const v2 z = {p2.y, -p2.x};
  return 0.5 * fabs(dot(p1, z));
}

void ro_cell_geometry(const rg_mesh_view* m, int ghost_kind, const double* box, double* volume, double* cm_xy,
                      double* cd_volume) {
  const int N = m->n_cells;
  for (int i = 0; i < N; ++i) {
    const int b = m->cell_face_offset[i], e1 = m->cell_face_offset[i + 1];
    /* VoronoiMesh.cpp:420-434 GetVolume: fan from the mesh point */
    const v2 c = point(m, i);
    double area = 0;
    for (int k = b; k < e1; ++k) {
      const int e = m->cell_faces[k];
      area += half_cross(vsub(vert0(m, e), c), vsub(vert1(m, e), c));
    }
    volume[i] = area;
    /* VoronoiMesh.cpp:436-451 CalcCellCM: fan from the first edge's first
     * vertex; physical_geometry.cpp:13-21 SlabSymmetry::calcVolume sums the
     * same triangles (triangle_area.cpp calc_triangle_area) in the same order */
    const v2 anchor = vert0(m, m->cell_faces[b]);
    v2 pc = {0, 0};
    double a2 = 0, vol = 0;
    for (int k = b + 1; k < e1; ++k) {
      const int e = m->cell_faces[k];
      const v2 f = vert0(m, e), s = vert1(m, e);
      const double t = half_cross(vsub(f, anchor), vsub(s, anchor));
      a2 += t;
      pc = vadd(pc, vscale(vadd(vadd(anchor, f), s), t / 3.));
      vol += half_cross(vsub(f, anchor), vsub(s, anchor));
    }
    cm_xy[2 * i] = pc.x / a2;
    cm_xy[2 * i + 1] = pc.y / a2;
    cd_volume[i] = vol;
  }
  /* VoronoiMesh.cpp:355-398 ghost CMs: periodic copies are shifted by the
   * ghost's offset from its source point; rigid-wall copies are reflected
   * (GetReflection, :316-330) about the box side they lie beyond */
  for (int g = 0; g < m->n_ghosts; ++g) {
    const int p = N + g, src = m->ghost_source[g];
    const v2 cs = {cm_xy[2 * src], cm_xy[2 * src + 1]};
    v2 r;
    if (ghost_kind == RG_GHOST_PERIODIC) {
      r = vadd(cs, vsub(point(m, p), point(m, src)));
    } else {
      const v2 q = point(m, p);
      r = cs;
      if (q.x > box[1]) {
        const v2 d = {2 * (box[1] - cs.x), 0};
        r = vadd(cs, d);
      } else if (q.y > box[3]) {
        const v2 d = {0, 2 * (box[3] - cs.y)};
        r = vadd(cs, d);
      } else if (q.x < box[0]) {
        const v2 d = {2 * (box[0] - cs.x), 0};
        r = vadd(cs, d);
      } else if (q.y < box[2]) {
        const v2 d = {0, 2 * (box[2] - cs.y)};
        r = vadd(cs, d);
      }
    }
    cm_xy[2 * p] = r.x;
    cm_xy[2 * p + 1] = r.y;
  }
}

/* ---------------- condition/action flux schemes ---------------- */

/* geometry.cpp normalize: v/abs(v) */
static v2 vnormalize(v2 v) { return vdiv(v, vabs(v)); }

static int has_sticker(const uint32_t* st, const rg_mesh_view* m, int p, int bit) {
  return st && bit >= 0 && ((st[orig(m, p)] >> bit) & 1u);
}

/* condition_action_sequence.cpp:228-289: (applies, aux) */
static int cas_condition(const rg_mesh_view* m, const ro_flux_rule* r, int e, const uint32_t* st, int* aux) {
  const int N = m->n_cells, a = fc0(m, e), b = fc1(m, e);
  *aux = 0;
  if (r->cond == 0) { /* IsBoundaryEdge, serial build */
    if (a < 0 || a >= N) return 1;
    if (b < 0 || b >= N) { *aux = 1; return 1; }
    return 0;
  }
  if (r->cond == 1) /* IsBulkEdge */
    return a >= 0 && b >= 0 && ((a < N && b < N) || orig(m, a) != orig(m, b));
  /* RegularSpecialEdge: exactly one side carries the sticker; aux = the second does */
  const int sa = has_sticker(st, m, a, r->sticker), sb = has_sticker(st, m, b, r->sticker);
  if (sa) return !sb;
  if (sb) { *aux = 1; return 1; }
  return 0;
}

/* condition_action_sequence.cpp:127-138 rigid_wall_states */
static void wall_states(prim s, v2 p, int aux, prim* l, prim* r) {
  if (aux) { *l = s; *r = reflect(s, p); }
  else { *r = s; *l = reflect(s, p); }
}

/* the wall frame of RigidWallFlux / FreeFlowFlux (:140-158, :186-204) */
static v2 wall_normal(const rg_mesh_view* m, int e, int aux, v2 p) {
  const v2 w = aux ? vsub(vert0(m, e), point(m, fc0(m, e))) : vsub(point(m, fc1(m, e)), vert0(m, e));
  return vnormalize(remove_parallel(w, p));
}

/* the tracer flux of one condition/action face: Mass times the tracers of
 * the cell (tcell, n_cells*nt) or LinearGaussImproved face value (tip, the
 * face's 2*nt) of the side the action takes, as the reference's
 * conserved_to_extensive forms it: tracers * Mass */
static void cas_tracer_flux(int nt, double mass, int first, int face_value, const double* tr, int ca, int cb,
                            const double* tip, double* out) {
  for (int j = 0; j < nt; ++j) {
    const double q = face_value ? tip[first ? j : nt + j] : tr[(size_t)(first ? ca : cb) * nt + j];
    out[j] = q * mass;
  }
}

int ro_cas_flux_tr(const rg_mesh_view* m, const double* cells, const double* tr, const double* ev, double g,
                   int order, const ro_lgi_params* lp, const ro_tracers* t, const ro_flux_rule* rules, int n_rules,
                   const uint32_t* st, double* fluxes, double* tfluxes, double* lag_ws, double* lag_ev,
                   ro_error* err) {
  const int nt = (t && tr && tfluxes) ? t->n : 0;
  const size_t E = (size_t)(m->n_faces > 0 ? m->n_faces : 1);
  double* ip = NULL;
  double* tip = NULL;
  int rc = 0;
  if (order == 2) {
    ip = (double*)malloc(sizeof(double) * 8 * E);
    if (nt > 0) {
      tip = (double*)malloc(sizeof(double) * 2 * (size_t)nt * E);
      rc = ro_lgi_tr(m, cells, tr, g, lp, t, NULL, ip, NULL, tip, err);
    } else {
      rc = ro_lgi(m, cells, g, lp, NULL, ip, err);
    }
  }
  for (int e = 0; e < m->n_faces && !rc; ++e) {
    const int a = fc0(m, e), b = fc1(m, e);
    int chosen = -1, aux = 0;
    for (int pass = 0; pass < 2 && chosen < 0; ++pass)
      for (int k = 0; k < n_rules && chosen < 0; ++k)
        if (rules[k].seq == pass && cas_condition(m, &rules[k], e, st, &aux)) chosen = k;
    if (chosen < 0) { /* condition_action_sequence_2.cpp:73 "Error in ConditionActionSequence" */
      set_err(err, RG_ERR_INVALID_ARGUMENT, 3, e, 0);
      rc = RG_ERR_INVALID_ARGUMENT;
      break;
    }
    const ro_flux_rule* r = &rules[chosen];
    const v2 p = vnormalize(vsub(vert1(m, e), vert0(m, e)));
    const v2 w = {ev[2 * e], ev[2 * e + 1]};
    const cc c0 = cell_at(cells, orig(m, a)), c1 = cell_at(cells, orig(m, b));
    const cc s0 = ip ? get_cc(ip + 8 * e) : c0, s1 = ip ? get_cc(ip + 8 * e + 4) : c1;
    int action = r->action;
    if (action == 5) {
      /* condition_action_sequence_2.cpp:232-249 Ratchet */
      const v2 nn = aux ? vsub(point(m, b), point(m, a)) : vsub(point(m, a), point(m, b));
      const cc sc = aux ? c0 : c1;
      const v2 vel = {sc.vx, sc.vy};
      action = dot(nn, vel) * (2 * (double)(r->in != 0) - 1) < 0 ? 2 : 4;
    }
    cons c;
    prim l, rr;
    v2 n;
    double v = 0;
    if (lag_ws) lag_ws[e] = 0;
    if (lag_ev) lag_ev[e] = 0;
    if (action == 6) {
      /* LagrangianFlux: CAS2's calc_parallel_normal (:17-27), the face speed,
       * WallsMassFlux (:300-312) choosing the solver, ws_ / edge_vel_ */
      const v2 pp = parallel(m, e);
      const int N = m->n_cells;
      const v2 nn = (a >= 0 && a < N) ? remove_parallel(vsub(vert0(m, e), point(m, a)), pp)
                                      : remove_parallel(vsub(point(m, b), vert0(m, e)), pp);
      const double speed = dot(nn, w) / vabs(nn);
      const int lag = orig(m, a) != orig(m, b);
      const int mf = lag ? (r->massflux & 1) : ((r->massflux >> 1) & 1);
      double energy = 0;
      rc = rotate_solve_rotate_back_lag(to_prim(g, s0), to_prim(g, s1), speed, mf, nn, pp, &c, &energy, e, err);
      if (rc) break;
      put_flux(fluxes + 4 * e, c);
      if (lag_ws) lag_ws[e] = lag ? energy : 0;
      if (lag_ev) lag_ev[e] = speed;
      /* convert_conserved_to_extensive (:29-40): the upwind face value */
      if (nt > 0)
        cas_tracer_flux(nt, c.m, c.m > 0, 1, tr, orig(m, a), orig(m, b), tip + (size_t)e * 2 * nt,
                        tfluxes + (size_t)e * nt);
      continue;
    }
    if (action == 0 || action == 3) {
      /* RegularFlux (condition_action_sequence.cpp:84-110), RegularFlux2
       * (condition_action_sequence_2.cpp:129-157) */
      n = vnormalize(vsub(point(m, b), point(m, a)));
      v = dot(n, w);
      l = to_prim(g, action == 0 ? c0 : s0);
      rr = to_prim(g, action == 0 ? c1 : s1);
    } else if (action == 1 || action == 4) {
      /* RigidWallFlux (:140-184), RigidWallFlux2 (:183-228) */
      n = wall_normal(m, e, aux, p);
      const cc sc = action == 1 ? (aux ? c0 : c1) : (aux ? s0 : s1);
      wall_states(to_prim(g, sc), p, aux, &l, &rr);
    } else {
      /* FreeFlowFlux (:186-220) */
      n = wall_normal(m, e, aux, p);
      l = rr = to_prim(g, aux ? c0 : c1);
    }
    rc = rotate_solve_rotate_back(l, rr, v, n, p, &c, e, err);
    if (rc) break;
    put_flux(fluxes + 4 * e, c);
    if (nt > 0) {
      /* RegularFlux: the upwind cell (condition_action_sequence.cpp:110-114);
       * RegularFlux2: the upwind face value (condition_action_sequence_2.cpp:156);
       * RigidWallFlux, FreeFlowFlux: the aux side's cell (:178, :221);
       * RigidWallFlux2: the aux side's face value (condition_action_sequence_2.cpp:221) */
      const int regular = action == 0 || action == 3, face_value = action == 3 || action == 4;
      cas_tracer_flux(nt, c.m, regular ? c.m > 0 : aux, face_value, tr, orig(m, a), orig(m, b),
                      tip ? tip + (size_t)e * 2 * nt : NULL, tfluxes + (size_t)e * nt);
    }
  }
  free(ip);
  free(tip);
  return rc;
}

int ro_cas_flux(const rg_mesh_view* m, const double* cells, const double* ev, double g, int order,
                const ro_lgi_params* lp, const ro_flux_rule* rules, int n_rules, const uint32_t* st,
                double* fluxes, double* lag_ws, double* lag_ev, ro_error* err) {
  return ro_cas_flux_tr(m, cells, NULL, ev, g, order, lp, NULL, rules, n_rules, st, fluxes, NULL, lag_ws, lag_ev,
                        err);
}

void ro_lagrangian_update_tr(const rg_mesh_view* m, const double* ws, const double* ev, double dt,
                             const double* areas, double* ext, double* tr_ext, int nt) {
  for (int i = 0; i < m->n_cells; ++i) {
    double dv = 0, dvw = 0;
    for (int k = m->cell_face_offset[i]; k < m->cell_face_offset[i + 1]; ++k) {
      const int e = m->cell_faces[k];
      const double area = areas ? areas[e] : edge_length(m, e);
      if (fc0(m, e) == i) {
        dv += area * dt * ev[e];
        dvw += area * dt * ws[e];
      } else {
        dv -= area * dt * ev[e];
        dvw -= area * dt * ws[e];
      }
    }
    const double V = m->cd_volume[i];
    const double a = (V + dv) / (V + dv + dvw);
    /* Extensive::operator*= (extensive.cpp:98-107): every component and tracer */
    for (int c = 0; c < 4; ++c) ext[4 * i + c] *= a;
    for (int j = 0; j < nt; ++j) tr_ext[(size_t)i * nt + j] *= a;
  }
}

void ro_lagrangian_update(const rg_mesh_view* m, const double* ws, const double* ev, double dt,
                          const double* areas, double* ext) {
  for (int i = 0; i < m->n_cells; ++i) {
    double dv = 0, dvw = 0;
    for (int k = m->cell_face_offset[i]; k < m->cell_face_offset[i + 1]; ++k) {
      const int e = m->cell_faces[k];
      const double area = areas ? areas[e] : edge_length(m, e);
      if (fc0(m, e) == i) {
        dv += area * dt * ev[e];
        dvw += area * dt * ws[e];
      } else {
        dv -= area * dt * ev[e];
        dvw -= area * dt * ws[e];
      }
    }
    const double V = m->cd_volume[i];
    const double a = (V + dv) / (V + dv + dvw);
    for (int c = 0; c < 4; ++c) ext[4 * i + c] *= a;
  }
}

int ro_step_cas(const rg_mesh_view* m, double* cells, double* ext, const double* ev, double g, double cfl,
                int order, const ro_lgi_params* lp, const ro_flux_rule* rules, int n_rules, const uint32_t* st,
                uint32_t frozen_mask, int lagrangian_update, double* dt_out, ro_error* err) {
  double dt;
  int rc = ro_cfl(m, cells, ev, g, cfl, &dt, err);
  if (rc) return rc;
  const size_t N = (size_t)m->n_cells;
  const size_t E = (size_t)(m->n_faces > 0 ? m->n_faces : 1);
  double* fl = (double*)malloc(sizeof(double) * 4 * E);
  double* ws = (double*)calloc(E, sizeof(double));
  double* lev = (double*)calloc(E, sizeof(double));
  double* old = (double*)malloc(sizeof(double) * 4 * N);
  memcpy(old, cells, sizeof(double) * 4 * N);
  rc = ro_cas_flux(m, cells, ev, g, order, lp, rules, n_rules, st, fl, ws, lev, err);
  if (!rc) rc = ro_extensive_update(m, fl, dt, ext, err);
  if (!rc && lagrangian_update) ro_lagrangian_update(m, ws, lev, dt, NULL, ext);
  if (!rc) {
    ro_tracers t;
    memset(&t, 0, sizeof t);
    t.entropy = -1;
    t.frozen_mask = frozen_mask;
    t.stickers = st;
    rc = ro_cell_update_tr(m, ext, NULL, old, NULL, g, &t, cells, NULL, err);
  }
  free(fl);
  free(ws);
  free(lev);
  free(old);
  if (dt_out) *dt_out = dt;
  return rc;
}

int ro_step_cas_tr(const rg_mesh_view* m, double* cells, double* ext, double* tr, double* tr_ext, const double* ev,
                   double g, double cfl, int order, const ro_lgi_params* lp, const ro_flux_rule* rules, int n_rules,
                   const ro_tracers* t, int lagrangian_update, double* dt_out, ro_error* err) {
  double dt;
  int rc = ro_cfl(m, cells, ev, g, cfl, &dt, err);
  if (rc) return rc;
  const int nt = t ? t->n : 0;
  const size_t N = (size_t)m->n_cells;
  const size_t E = (size_t)(m->n_faces > 0 ? m->n_faces : 1);
  double* fl = (double*)malloc(sizeof(double) * 4 * E);
  double* tfl = (double*)malloc(sizeof(double) * E * (nt > 0 ? nt : 1));
  double* ws = (double*)calloc(E, sizeof(double));
  double* lev = (double*)calloc(E, sizeof(double));
  double* old = (double*)malloc(sizeof(double) * 4 * N);
  double* old_tr = (double*)malloc(sizeof(double) * N * (nt > 0 ? nt : 1));
  memcpy(old, cells, sizeof(double) * 4 * N);
  if (nt > 0) memcpy(old_tr, tr, sizeof(double) * N * nt);
  rc = ro_cas_flux_tr(m, cells, tr, ev, g, order, lp, t, rules, n_rules, t ? t->stickers : NULL, fl, tfl, ws, lev,
                      err);
  if (!rc) rc = ro_extensive_update(m, fl, dt, ext, err);
  if (!rc) ro_extensive_update_tr(m, tfl, nt, dt, tr_ext);
  if (!rc && lagrangian_update) ro_lagrangian_update_tr(m, ws, lev, dt, NULL, ext, tr_ext, nt);
  if (!rc) rc = ro_cell_update_tr(m, ext, tr_ext, old, old_tr, g, t, cells, tr, err);
  free(fl);
  free(tfl);
  free(ws);
  free(lev);
  free(old);
  free(old_tr);
  if (dt_out) *dt_out = dt;
  return rc;
}

/* physical_geometry.cpp:44-60 Axis and change_coordinate: (along, |across|) */
typedef struct { v2 origin, dir; } axis2;
static v2 change_coordinate(v2 v, axis2 a) {
  const v2 d = vsub(v, a.origin);
  const v2 z = {a.dir.y, -a.dir.x};
  v2 r = {dot(d, a.dir), fabs(dot(d, z))};
  return r;
}
/* :75-82 calc_cone_segment_volume (pow(x,2.) is x*x) */
static double cone_segment(v2 p1, v2 p2, axis2 a) {
  const v2 q1 = change_coordinate(p1, a), q2 = change_coordinate(p2, a);
  return (RO_PI / 3.) * (q2.x - q1.x) * (q1.y * q1.y + q2.y * q2.y + q1.y * q2.y);
}

void ro_cyl_geometry(const rg_mesh_view* m, const double* origin, const double* direction, double* areas,
                     double* volumes) {
  const v2 dd = {direction[0], direction[1]};
  axis2 a;
  a.origin.x = origin[0];
  a.origin.y = origin[1];
  a.dir = vdiv(dd, vabs(dd)); /* physical_geometry.cpp:40-42 */
  for (int e = 0; e < m->n_faces; ++e) {
    /* :66-71 calcArea */
    const v2 p1 = change_coordinate(vert0(m, e), a), p2 = change_coordinate(vert1(m, e), a);
    const double dy = p2.y - p1.y, dx = p2.x - p1.x;
    areas[e] = RO_PI * (p1.y + p2.y) * sqrt(dy * dy + dx * dx);
  }
  for (int i = 0; i < m->n_cells; ++i) {
    /* :94-104 calcVolume over the cell's edges, :84-92 calc_triangular_ring_volume */
    const int b = m->cell_face_offset[i], e1 = m->cell_face_offset[i + 1];
    const v2 anchor = vert0(m, m->cell_faces[b]);
    double res = 0;
    for (int k = b + 1; k < e1; ++k) {
      const int e = m->cell_faces[k];
      const v2 f = vert0(m, e), s2 = vert1(m, e);
      res += fabs(cone_segment(anchor, f, a) + cone_segment(f, s2, a) + cone_segment(s2, anchor, a));
    }
    volumes[i] = res;
  }
}

void ro_extensive_update_areas(const rg_mesh_view* m, const double* fluxes, const double* areas, double dt,
                               double* ext) {
  const int N = m->n_cells;
  for (int e = 0; e < m->n_faces; ++e) {
    const double s = dt * areas[e];
    const double dm = fluxes[4 * e] * s, de = fluxes[4 * e + 1] * s;
    const double dx = fluxes[4 * e + 2] * s, dy = fluxes[4 * e + 3] * s;
    const int a = fc0(m, e), b = fc1(m, e);
    if (a >= 0 && a < N) {
      ext[4 * a] -= dm;
      ext[4 * a + 1] -= de;
      ext[4 * a + 2] -= dx;
      ext[4 * a + 3] -= dy;
    }
    if (b >= 0 && b < N) {
      ext[4 * b] += dm;
      ext[4 * b + 1] += de;
      ext[4 * b + 2] += dx;
      ext[4 * b + 3] += dy;
    }
  }
}

int ro_step_areas(const rg_mesh_view* m, double* cells, double* ext, const double* ev, double g, double cfl,
                  int order, const ro_lgi_params* lp, const double* areas, double* dt_out, ro_error* err) {
  double dt;
  int st = ro_cfl(m, cells, ev, g, cfl, &dt, err);
  if (st) return st;
  double* fl = (double*)malloc(sizeof(double) * 4 * (size_t)(m->n_faces > 0 ? m->n_faces : 1));
  st = order == 1 ? ro_simple_flux(m, cells, ev, g, fl, err) : ro_modular_flux(m, cells, ev, g, lp, fl, err);
  if (!st) ro_extensive_update_areas(m, fl, areas, dt, ext);
  if (!st) st = ro_cell_update(m, ext, g, cells, err);
  free(fl);
  if (dt_out) *dt_out = dt;
  return st;
}

/* round_cells.cpp:69-81 calc_dw (hot form) */
static v2 round_dw(const rg_mesh_view* m, const double* cells, double g, const ro_motion* mo, int i) {
  const v2 r = point(m, i), s = cmof(m, i);
  const double d = vabs(vsub(s, r));
  const double R = width(m, i);
  const v2 zero = {0, 0};
  if (d < 0.9 * mo->eta * R) return zero;
  const v2 v = {cells[4 * i + 2], cells[4 * i + 3]};
  const double c = smax(dp2c(g, cells[4 * i], cells[4 * i + 1]), vabs(v));
  return vdiv(vscale(vsub(s, r), mo->chi * c), R);
}

/* round_cells.cpp:83-103 calc_dw (cold form, with dt); the neighbour test
 * compares the neighbour's id with the neighbour count, as the reference does;
 * ids past the real cells, which the reference would read out of range, are
 * left out */
static v2 round_dw_cold(const rg_mesh_view* m, const double* cells, double g, const ro_motion* mo, int i,
                        double dt) {
  const v2 r = point(m, i), s = cmof(m, i);
  const double d = vabs(vsub(s, r));
  const double R = width(m, i);
  const v2 zero = {0, 0};
  if (d < 0.9 * mo->eta * R) return zero;
  const int b = m->cell_face_offset[i], nn = m->cell_face_offset[i + 1] - b;
  const v2 v = {cells[4 * i + 2], cells[4 * i + 3]};
  double cs = smax(vabs(v), dp2c(g, cells[4 * i], cells[4 * i + 1]));
  for (int k = 0; k < nn; ++k) {
    const int e = m->cell_faces[b + k];
    const int nb = fc0(m, e) != i ? fc0(m, e) : fc1(m, e);
    if (orig(m, nb) == i || nb > nn || nb >= m->n_cells) continue;
    const v2 vn = {cells[4 * nb + 2], cells[4 * nb + 3]};
    cs = smax(cs, dp2c(g, cells[4 * nb], cells[4 * nb + 1]));
    cs = smax(cs, vabs(vn));
  }
  const double c_dt = d / dt;
  return vdiv(vscale(vsub(s, r), mo->chi * smin(c_dt, cs)), R);
}

void ro_point_velocities(const rg_mesh_view* m, const double* cells, double g, const ro_motion* mo, double* pv) {
  for (int i = 0; i < m->n_cells; ++i) {
    v2 w = {0, 0};
    if (mo->kind >= 1) { /* lagrangian.cpp:3-13 */
      w.x = cells[4 * i + 2];
      w.y = cells[4 * i + 3];
    }
    if (mo->kind == 2 && !mo->cold) w = vadd(w, round_dw(m, cells, g, mo, i)); /* round_cells.cpp:105-119 */
    pv[2 * i] = w.x;
    pv[2 * i + 1] = w.y;
  }
}

/* round_cells.cpp:15-63 CorrectPointsOverShoot for one point */
static v2 overshoot(const rg_mesh_view* m, const ro_motion* mo, int i, double dt, v2 v) {
  const v2 p = point(m, i);
  const double R = width(m, i);
  const double inv_dt = 1.0 / dt;
  const double L = mo->box[0], Rt = mo->box[1], D = mo->box[2], U = mo->box[3];
  if ((v.x * dt * 2 + p.x) > Rt) {
    double f = 0.25 * (Rt - p.x) * inv_dt / vabs(v);
    if (R * 0.1 > (Rt - p.x)) f *= -0.1;
    v = vscale(v, f);
  }
  if ((v.x * dt * 2 + p.x) < L) {
    double f = 0.25 * (p.x - L) * inv_dt / vabs(v);
    if (R * 0.1 > (p.x - L)) f *= -0.1;
    v = vscale(v, f);
  }
  if ((v.y * dt * 2 + p.y) > U) {
    double f = 0.25 * (U - p.y) * inv_dt / vabs(v);
    if (R * 0.1 > (U - p.y)) f *= -0.1;
    v = vscale(v, f);
  }
  if ((v.y * dt * 2 + p.y) < D) {
    double f = 0.25 * (p.y - D) * inv_dt / vabs(v);
    if (R * 0.1 > (p.y - D)) f *= -0.1;
    v = vscale(v, f);
  }
  return v;
}

/* round_cells.cpp:121-134 RoundCells::ApplyFix (point_motion.cpp:5-9: the
 * wrapped motion leaves the velocities) */
void ro_apply_fix(const rg_mesh_view* m, const double* cells, double g, const ro_motion* mo, double dt, double* pv) {
  if (mo->kind != 2) return;
  for (int i = 0; i < m->n_cells; ++i) {
    v2 w = {pv[2 * i], pv[2 * i + 1]};
    if (mo->cold) w = vadd(w, round_dw_cold(m, cells, g, mo, i, dt));
    if (mo->correct_overshoot) w = overshoot(m, mo, i, dt, w);
    pv[2 * i] = w.x;
    pv[2 * i + 1] = w.y;
  }
}

/* VoronoiMesh.cpp:146-151 CalcFaceVelocity (pow(x,2) is x*x) */
static v2 face_velocity(v2 wl, v2 wr, v2 rl, v2 rr, v2 f) {
  const v2 mid = vdiv(vadd(rr, rl), 2);
  const v2 dr = vsub(rr, rl);
  const double a = vabs(dr);
  const v2 wp = vdiv(vscale(dr, dot(vsub(wl, wr), vsub(f, mid))), a * a);
  return vadd(vscale(vadd(wl, wr), 0.5), wp);
}

/* stationary_box.cpp:20-40 (0 on a face between a point and its own copy)
 * and periodic_edge_velocities.cpp:5-21; a ghost takes its source point's
 * velocity (StationaryBox indexes the point velocities with the ghost id,
 * which only a face of a point and its own copy could reach) */
void ro_edge_velocities(const rg_mesh_view* m, const ro_motion* mo, const double* pv, double* ev) {
  for (int e = 0; e < m->n_faces; ++e) {
    const int a = fc0(m, e), b = fc1(m, e);
    const int oa = orig(m, a), ob = orig(m, b);
    v2 w = {0, 0};
    if (mo->edges == 1 || oa != ob) {
      const v2 wl = {pv[2 * oa], pv[2 * oa + 1]}, wr = {pv[2 * ob], pv[2 * ob + 1]};
      w = face_velocity(wl, wr, point(m, a), point(m, b), centroid(m, e));
    }
    ev[2 * e] = w.x;
    ev[2 * e + 1] = w.y;
  }
}

/* ========================================================================
 * 3D first-order path (HDSim3D on a CubeGrid-like packed mesh)
 * ======================================================================== */

typedef struct { double x, y, z; } v3;
typedef struct { double d, p; v3 v; } cc3;
typedef struct { double m; v3 mom; double en; } cons3;

/* Vector3D.cpp: abs, ScalarProd, operator*(double, Vector3D) (v.x*d), /, -, + */
static double v3abs(v3 v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
static double v3dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 v3scale(double d, v3 v) { v3 r = {v.x * d, v.y * d, v.z * d}; return r; }
static v3 v3div(v3 v, double d) { v3 r = {v.x / d, v.y / d, v.z / d}; return r; }
static v3 v3sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static v3 v3add(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }

static cc3 cell3(const double* c, int i) {
  cc3 r = {c[5 * i], c[5 * i + 1], {c[5 * i + 2], c[5 * i + 3], c[5 * i + 4]}};
  return r;
}
static v3 normal3(const rg_mesh3d_view* m, int f) {
  v3 n = {m->face_normal[3 * f], m->face_normal[3 * f + 1], m->face_normal[3 * f + 2]};
  return v3div(n, v3abs(n)); /* FirstOrderHydroFlux.cpp:11-14 normalize */
}

/* FirstOrderHydroFlux.cpp:32-40 calc_primitive: (d, p, (v.n, |v - (v.n)n|), e, c) */
static prim prim3(double g, cc3 c, v3 n) {
  const double sp = v3dot(c.v, n);
  prim r;
  r.d = c.d;
  r.p = c.p;
  r.vx = sp;
  r.vy = v3abs(v3sub(c.v, v3scale(sp, n)));
  r.e = dp2e(g, c.d, c.p);
  r.c = dp2c(g, c.d, c.p);
  return r;
}

/* FirstOrderHydroFlux.cpp:16-30 GetParallel */
static v3 parallel3(v3 vel, v3 n) {
  v3 par = v3sub(vel, v3scale(v3dot(vel, n), n));
  const double p = v3abs(par);
  const double v = v3abs(vel);
  if (1e-9 > fabs(v - 0)) return par;
  if (p < 1e-8 * v)
    par = v3div(par, v);
  else
    par = v3div(par, p);
  return par;
}

/* Vector3D.cpp:203-206 Reflect: v - 2*ScalarProd(v,n)*n/pow(abs(n),2) (pow(x,2) folds to x*x) */
static v3 reflect3(v3 v, v3 n) {
  const double s = 2 * v3dot(v, n);
  const double a = v3abs(n);
  return v3sub(v, v3div(v3scale(s, n), a * a));
}

static cons3 rebuild(cons sol, v3 n, v3 par) {
  cons3 r;
  r.m = sol.m;
  r.mom = v3add(v3scale(sol.mx, n), v3scale(sol.my, par));
  r.en = sol.en;
  return r;
}

/* FirstOrderHydroFlux.cpp:98-114 operator(), :42-66 CalcRigidWall, :68-88 CalcSingleFluxInBulk */
int ro3_flux(const rg_mesh3d_view* m, const double* cells, const double* fvel, double gamma, double* fluxes,
             ro_error* err) {
  for (int f = 0; f < m->n_faces; ++f) {
    const int a = m->face_cells[2 * f], b = m->face_cells[2 * f + 1];
    const v3 n = normal3(m, f);
    cons sol;
    cons3 res;
    if (a < 0 || b < 0) {
      const int real_first = a >= 0;
      const cc3 real = cell3(cells, real_first ? a : b);
      const prim preal = prim3(gamma, real, n);
      const v3 par = parallel3(real.v, n);
      cc3 other = real;
      other.v = reflect3(real.v, n);
      const prim pghost = prim3(gamma, other, n);
      const double fv = 0;
      const int st = real_first ? hllc(preal, pghost, fv, &sol, f, err) : hllc(pghost, preal, fv, &sol, f, err);
      if (st) return st;
      res = rebuild(sol, n, par);
    } else {
      v3 w = {0, 0, 0};
      if (fvel) {
        w.x = fvel[3 * f];
        w.y = fvel[3 * f + 1];
        w.z = fvel[3 * f + 2];
      }
      const double fv = v3dot(w, n);
      const cc3 ca = cell3(cells, a), cb = cell3(cells, b);
      const int st = hllc(prim3(gamma, ca, n), prim3(gamma, cb, n), fv, &sol, f, err);
      if (st) return st;
      const cc3 donor = sol.m > 0 ? ca : cb;
      res = rebuild(sol, n, parallel3(donor.v, n));
    }
    double* o = fluxes + 5 * f;
    o[0] = res.m;
    o[1] = res.mom.x;
    o[2] = res.mom.y;
    o[3] = res.mom.z;
    o[4] = res.en;
  }
  return 0;
}

/* hdsim_3d.cpp:63-76 update_extensive: delta = dt*area*flux per face, in face order */
void ro3_extensive_update(const rg_mesh3d_view* m, const double* fluxes, double dt, double* ext) {
  for (int f = 0; f < m->n_faces; ++f) {
    const double s = dt * m->face_area[f];
    const double* fl = fluxes + 5 * f;
    double d[5];
    for (int q = 0; q < 5; ++q) d[q] = s * fl[q];
    const int a = m->face_cells[2 * f], b = m->face_cells[2 * f + 1];
    if (a >= 0)
      for (int q = 0; q < 5; ++q) ext[5 * a + q] -= d[q];
    if (b >= 0)
      for (int q = 0; q < 5; ++q) ext[5 * b + q] += d[q];
  }
}

/* hdsim_3d.cpp:78-104 AllCellsUpdater (extensive/volume) with DefaultCellUpdater
 * (default_cell_updater.cpp:5-14) and IdealGas::de2p (ideal_gas.cpp:18-23) */
int ro3_cell_update(const rg_mesh3d_view* m, const double* ext, double gamma, double* cells, ro_error* err) {
  for (int i = 0; i < m->n_cells; ++i) {
    const double V = m->volume[i];
    const double* e = ext + 5 * i;
    const double mass = e[0] / V;
    const v3 mom = {e[1] / V, e[2] / V, e[3] / V};
    const double en = e[4] / V;
    const double density = mass;
    const v3 vel = v3div(mom, density);
    const double thermal = en - 0.5 * density * v3dot(vel, vel);
    const double eint = thermal / density;
    if (eint < 0) {
      set_err(err, RG_ERR_NEGATIVE_ENERGY, 5, i, eint);
      return RG_ERR_NEGATIVE_ENERGY;
    }
    double* c = cells + 5 * i;
    c[0] = density;
    c[1] = (gamma - 1) * eint * density;
    c[2] = vel.x;
    c[3] = vel.y;
    c[4] = vel.z;
  }
  return 0;
}

/* extensive_generator.cpp:3-28: volume * (d, d*v, d*(0.5*v.v + e)) */
void ro3_init_extensives(const rg_mesh3d_view* m, const double* cells, double gamma, double* ext) {
  for (int i = 0; i < m->n_cells; ++i) {
    const cc3 c = cell3(cells, i);
    const double V = m->volume[i];
    const v3 mom = v3scale(c.d, c.v);
    const double en = c.d * (0.5 * v3dot(c.v, c.v) + dp2e(gamma, c.d, c.p));
    double* e = ext + 5 * i;
    e[0] = V * c.d;
    e[1] = mom.x * V;
    e[2] = mom.y * V;
    e[3] = mom.z * V;
    e[4] = V * en;
  }
}

/* CourantFriedrichsLewy.cpp:23-46: cfl * min width/(|v| + c) */
double ro3_cfl(const rg_mesh3d_view* m, const double* cells, double gamma, double cfl) {
  double best = 0;
  for (int i = 0; i < m->n_cells; ++i) {
    const cc3 c = cell3(cells, i);
    const double b = m->width[i] / (v3abs(c.v) + dp2c(gamma, c.d, c.p));
    best = i == 0 ? b : smin(best, b);
  }
  return cfl * best;
}

int ro3_step(const rg_mesh3d_view* m, double* cells, double* ext, double gamma, double cfl, double* dt_out,
             ro_error* err) {
  const double dt = ro3_cfl(m, cells, gamma, cfl);
  double* fl = (double*)malloc(sizeof(double) * 5 * (size_t)(m->n_faces > 0 ? m->n_faces : 1));
  if (!fl) return RG_ERR_OUT_OF_MEMORY;
  int st = ro3_flux(m, cells, NULL, gamma, fl, err);
  if (!st) {
    ro3_extensive_update(m, fl, dt, ext);
    st = ro3_cell_update(m, ext, gamma, cells, err);
  }
  free(fl);
  *dt_out = dt;
  return st;
}

