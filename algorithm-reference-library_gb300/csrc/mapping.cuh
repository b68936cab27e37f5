// Row mapping shared by the gridding, weighting and conversion kernels:
// uvw (wavelengths) and frequency -> grid pixel, sub-pixel kernel index,
// w-plane and channel, with integer results identical to NumPy's.
#pragma once
#include "common.cuh"

namespace arlgpu {

// ---------------------------------------------------------------------------
// Exact FP64 linear-axis transforms in numpy's operation order.
//   world2pix0(x) = ((x - crval) / cdelt + crpix) - 1
//   pix2world0(p) = ((p + 1) - crpix) * cdelt + crval
// Each operation is rounded on its own (no FMA contraction).  The division is
// first done as a multiply by the rounded reciprocal; when the result lies
// within a few ulps of the rounding boundary that decides the integer index
// (a half-integer for round-half-even, an integer for floor) the exact IEEE
// division recomputes it, so the index always equals numpy's.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double w2p_tail(double q, const arlgpu_axis &a) {
  return __dsub_rn(__dadd_rn(q, a.crpix), 1.0);
}
__device__ __forceinline__ double w2p_fast(double x, const arlgpu_axis &a, double rcp) {
  return w2p_tail(__dmul_rn(__dsub_rn(x, a.crval), rcp), a);
}
__device__ __forceinline__ double w2p_exact(double x, const arlgpu_axis &a) {
  return w2p_tail(__ddiv_rn(__dsub_rn(x, a.crval), a.cdelt), a);
}
__device__ __forceinline__ double p2w(double p, const arlgpu_axis &a) {
  return __dadd_rn(__dmul_rn(__dsub_rn(__dadd_rn(p, 1.0), a.crpix), a.cdelt), a.crval);
}
__device__ __forceinline__ double near_tol(double p) { return 1e-11 * (1.0 + fabs(p)); }

// numpy.round(world2pix0(x))
__device__ __forceinline__ double round_w2p(double x, const arlgpu_axis &a, double rcp) {
  double p = w2p_fast(x, a, rcp);
  double f = p - floor(p);
  if (fabs(f - 0.5) < near_tol(p)) p = w2p_exact(x, a);
  return rint(p);
}
// numpy.floor(world2pix0(x))
__device__ __forceinline__ double floor_w2p(double x, const arlgpu_axis &a, double rcp) {
  double p = w2p_fast(x, a, rcp);
  double f = p - rint(p);
  if (fabs(f) < near_tol(p)) p = w2p_exact(x, a);
  return floor(p);
}

// Support of plane z: plane_support[z] clamped to an even value in [2, S].
__device__ __forceinline__ int plane_sz(const Geom &g, int zc) {
  if (!g.plane_support) return g.S;
  int sz = g.plane_support[zc];
  sz = sz < 2 ? 2 : (sz > g.S ? g.S : sz);
  return sz & ~1;
}

struct Mapped {
  int32_t pu, pv, uf, vf, zg, zc, ch;
  bool ok;
};

// round(world2pix0(x)) through one FMA, falling back to the exact sequence
// when the fast value lies within tol of a half-integer.  Both the fast and
// NumPy's value are within a few ulps of x / cdelt + crpix - 1; tol is ~45 ulps.
__device__ __forceinline__ double round_w2p_fma(double x, const arlgpu_axis &a, double rcp) {
  const double p = fma(__dsub_rn(x, a.crval), rcp, a.crpix - 1.0);
  const double r = rint(p);
  if (0.5 - fabs(p - r) < 1e-14 * (fabs(p) + fabs(a.crpix) + 2.0)) return rint(w2p_exact(x, a));
  return r;
}

// Exact NumPy sequence for the u (or v) axis: (pixel, sub-pixel offset).
__device__ __forceinline__ void map_axis_exact(double x, const arlgpu_axis &ga, double rcp_g, const arlgpu_axis &ca,
                                               double rcp_c, double *pix, double *sub) {
  *pix = round_w2p(x, ga, rcp_g);
  *sub = floor_w2p(__dsub_rn(x, p2w(*pix, ga)), ca, rcp_c);
}

// The seven mapped indices of one row, as doubles, before any range check.
struct RawMap {
  double pu, pv, uf, vf, zg, zc, ch;
};

// Nearest-plane index with a tolerance fixed per axis on the host (valid for
// |P| < Plim, which covers every in-range index): the exact sequence when the
// fast value is within tol of a half-integer or beyond Plim.
__device__ __forceinline__ double round_w2p_tol(double x, const arlgpu_axis &a, double rcp, double Plim,
                                                double tol) {
  const double p = fma(__dsub_rn(x, a.crval), rcp, a.crpix - 1.0);
  const double r = rint(p);
  if (fabs(p) < Plim && fabs(p - r) < 0.5 - tol) return r;
  return rint(w2p_exact(x, a));
}

// Pixel and sub-pixel index of one axis from X = P * O (power-of-two O): away
// from integers of X, rint(P) = floor((floor(X) + O/2) / O) and the sub-pixel
// index is the remainder.  Returns false when X is within tol of an integer or
// beyond Xlim (the caller then takes the exact sequence).
__device__ __forceinline__ bool map_axis_x(double x, double rO, double cO, double Xlim, double tol, int O,
                                           int log2O, double *pix, double *sub) {
  const double X = fma(x, rO, cO);
  if (!(fabs(X) < Xlim)) return false;
  const double n = floor(X), fr = X - n;
  if (fr < tol || fr > 1.0 - tol) return false;
  const int a = (int)n + (O >> 1);
  const int pu = a >> log2O;  // arithmetic shift: floor division by O
  *pix = (double)pu;
  *sub = (double)(a - (pu << log2O));
  return true;
}

__device__ __forceinline__ RawMap map_raw(double u, double v, double w, double f, const Geom &g) {
  RawMap r;
  bool exact = !g.fast_uv;
  if (!exact && g.pow2O) {
    exact = !(map_axis_x(u, g.rOu, g.cOu, g.Xlim_u, g.tolX_u, g.O, g.log2O, &r.pu, &r.uf) &&
              map_axis_x(v, g.rOv, g.cOv, g.Xlim_v, g.tolX_v, g.O, g.log2O, &r.pv, &r.vf));
  } else if (!exact) {
    // One-FMA fast path (valid when crval == 0 on UU, VV, DUU, DVV and the cf's
    // DUU / DVV cdelt is the grid cdelt / O; the host checks this).  With
    // P = u / cdelt + crpix - 1, the nearest pixel is rint(P) and the sub-pixel
    // index is floor((P - pixel) O + O // 2); both fast values are within
    // ~O |P| 1e-16 of NumPy's, so any result within 1e-14 O (|P| + 2) of a
    // rounding boundary goes to the exact sequence instead.
    const double Pu = fma(u, g.rcp_gu, g.gu.crpix - 1.0), Pv = fma(v, g.rcp_gv, g.gv.crpix - 1.0);
    r.pu = rint(Pu);
    r.pv = rint(Pv);
    const double Qu = fma(Pu - r.pu, (double)g.O, g.cdu.crpix - 1.0);
    const double Qv = fma(Pv - r.pv, (double)g.O, g.cdv.crpix - 1.0);
    r.uf = floor(Qu);
    r.vf = floor(Qv);
    const double tu = 1e-14 * (fabs(Pu) + 2.0), tv = 1e-14 * (fabs(Pv) + 2.0);
    const double tqu = tu * g.O, tqv = tv * g.O;
    exact = (0.5 - fabs(Pu - r.pu) < tu) || (0.5 - fabs(Pv - r.pv) < tv) || (Qu - r.uf < tqu) ||
            (r.uf + 1.0 - Qu < tqu) || (Qv - r.vf < tqv) || (r.vf + 1.0 - Qv < tqv);
  }
  if (exact) {
    map_axis_exact(u, g.gu, g.rcp_gu, g.cdu, g.rcp_cdu, &r.pu, &r.uf);
    map_axis_exact(v, g.gv, g.rcp_gv, g.cdv, g.rcp_cdv, &r.pv, &r.vf);
  }
  r.zg = round_w2p_tol(w, g.gw, g.rcp_gw, g.Plim_w, g.tol_w);
  r.zc = round_w2p_tol(w, g.cz, g.rcp_cz, g.Plim_z, g.tol_z);
  r.ch = round_w2p_tol(f, g.gf, g.rcp_gf, g.Plim_f, g.tol_f);
  return r;
}

// Fixed-point view of a double with 20 fraction bits: for |X| < 2^31,
// y = X + 1.5 2^32 lies in [2^32, 2^33) where the ulp is 2^-20, so y's bit
// pattern minus that of 1.5 2^32 is X * 2^20 rounded to an integer.  One FP64
// add replaces a floor, a subtraction, comparisons and a conversion; the
// range test is y's exponent field (false for |X| >= 2^31 and NaN).
__device__ __forceinline__ bool fix20(double X, long long *F) {
  const long long b = __double_as_longlong(__dadd_rn(X, 6442450944.0));
  *F = b - 0x41F8000000000000LL;
  return (b >> 52) == 0x41F;
}

// Pixel and sub-pixel index of one axis from X = P * O (power-of-two O), as
// map_axis_x, with the integer-boundary test in fixed point: the fraction of
// X rounded to 2^-20 lies at least tq units from an integer, so X and NumPy's
// value (within tol of X) have the same floor.  Beyond the range where tol is
// valid (|X| >= Xlim) the index is out of the grid whichever way it rounds,
// so no separate range test is needed.
__device__ __forceinline__ bool fix_axis_x(double x, double rO, double cO, int tq, int O, int log2O, int *pix,
                                           int *sub) {
  long long F;
  if (!fix20(fma(x, rO, cO), &F)) return false;
  const int fr = (int)(F & 0xFFFFF);
  if (fr < tq || fr > (1 << 20) - tq) return false;
  const long long a = (F >> 20) + (O >> 1);
  const long long pl = a >> log2O;
  *pix = (int)max(min(pl, 0x3fffffffLL), -0x3fffffffLL);
  *sub = (int)(a - (pl << log2O));
  return true;
}

// Nearest-plane index as round_w2p_tol, with the half-integer test in fixed
// point (F = (P + 1/2) 2^20: the index is F >> 20 when F's fraction is at
// least tq units from an integer).
__device__ __forceinline__ bool fix_round(double x, const arlgpu_axis &a, double rcp, int tq, int *idx) {
  long long F;
  if (!fix20(fma(__dsub_rn(x, a.crval), rcp, a.crpix - 1.0), &F)) return false;
  F += 1LL << 19;
  const int fr = (int)(F & 0xFFFFF);
  if (fr < tq || fr > (1 << 20) - tq) return false;
  *idx = (int)(F >> 20);
  return true;
}

// Nearest-plane index of one axis in [0, n), or -1 outside: the fixed-point
// decision, and NumPy's exact sequence for that axis alone where the value
// lies within the tolerance of a half-integer.  Whole sets of rows can sit on
// such a tie: with an even number of w slices centred on w = 0, every row of
// a coplanar array at transit (w = 0 up to rounding) does.
__device__ __forceinline__ int plane_index(double x, const arlgpu_axis &a, double rcp, int tq, int n) {
  int idx;
  if (fix_round(x, a, rcp, tq, &idx)) return idx >= 0 && idx < n ? idx : -1;
  const double p = rint(w2p_exact(x, a));  // range test in double: no wrap when narrowed
  return p >= 0.0 && p < (double)n ? (int)p : -1;
}

__device__ __forceinline__ Mapped map_row(double u, double v, double w, double f, const Geom &g) {
  Mapped m;
  bool ok;
  int pu, pv, uf, vf, zg, zc, ch;
  if (g.fixmap && fix_axis_x(u, g.rOu, g.cOu, g.tq_u, g.O, g.log2O, &pu, &uf) &&
      fix_axis_x(v, g.rOv, g.cOv, g.tq_v, g.O, g.log2O, &pv, &vf)) {
    // uf, vf lie in [0, O) by construction
    zg = g.skip_zg ? 0 : plane_index(w, g.gw, g.rcp_gw, g.tq_w, g.nw);
    zc = g.skip_zc ? 0 : plane_index(w, g.cz, g.rcp_cz, g.tq_z, g.nz);
    ch = plane_index(f, g.gf, g.rcp_gf, g.tq_f, min(g.nchan, g.cf_nchan));
    ok = pu >= 0 && pu < g.nx && pv >= 0 && pv < g.ny && zg >= 0 && zc >= 0 && ch >= 0;
  } else {
    const RawMap r = map_raw(u, v, w, f, g);
    // Range checks in double so huge values cannot wrap when narrowed.
    ok = r.pu >= 0.0 && r.pu < g.nx && r.pv >= 0.0 && r.pv < g.ny && r.uf >= 0.0 && r.uf < g.O && r.vf >= 0.0 &&
         r.vf < g.O && r.zg >= 0.0 && r.zg < g.nw && r.zc >= 0.0 && r.zc < g.nz && r.ch >= 0.0 && r.ch < g.nchan &&
         r.ch < g.cf_nchan;
    pu = ok ? (int32_t)r.pu : 0;
    pv = ok ? (int32_t)r.pv : 0;
    uf = ok ? (int32_t)r.uf : 0;
    vf = ok ? (int32_t)r.vf : 0;
    zg = ok ? (int32_t)r.zg : 0;
    zc = ok ? (int32_t)r.zc : 0;
    ch = ok ? (int32_t)r.ch : 0;
  }
  m.pu = ok ? pu : -1;
  m.pv = ok ? pv : -1;
  m.uf = ok ? uf : 0;
  m.vf = ok ? vf : 0;
  m.zg = ok ? zg : 0;
  m.zc = ok ? zc : 0;
  m.ch = ok ? ch : 0;
  if (ok) {
    int h = plane_sz(g, m.zc) >> 1;
    ok = (m.pu - h >= 0) && (m.pu + h <= g.nx) && (m.pv - h >= 0) && (m.pv + h <= g.ny);
  }
  m.ok = ok;
  return m;
}

__device__ __forceinline__ uint32_t bin_of(int ch, int zg, int pu, int pv, const Geom &g) {
  return (((uint32_t)ch * g.nw + zg) * g.ntv + pv / g.T) * g.ntu + pu / g.T;
}

}  // namespace arlgpu
