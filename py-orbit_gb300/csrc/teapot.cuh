// TEAPOT symplectic maps as per-particle device functions.
//
// Each map restates one function of src/teapot/teapotbase.cc (cited per
// case).  The per-element constants the reference computes once per call
// (matrix elements, 1/factorial, cos/sin of the element angle) are computed
// on the host in the same way (compile_op in teapot.cu) and carried in
// DevOp::c; the per-particle arithmetic runs here in FP64 with fused
// multiply-add allowed.  Per particle, dp_p = dE/(p*beta) and
// KNL = 1/(1+dp_p) are computed once and reused by every map until a map
// changes dE, which gives exactly the values each map would recompute.
#pragma once

#include "common.cuh"
#include "softf64.cuh"

namespace orbit {

struct DevOp {
  int code, i0, i1, i2;
  double c[12];
};

struct MapCtx {
  double dp_p_coeff;  // 1/(p*beta)   (e.g. teapotbase.cc:168)
  double gamma2i;     // 1/gamma^2    (teapotbase.cc:167)
  double charge;      // bunch charge
};

struct Part {
  double x, xp, y, yp, z, dE;
  double dp_p, knl;
  bool knl_ok;
};

// Every operation of the maps below is written out (fma, dmul<S>, __dadd_rn,
// __dsub_rn), so that no kernel contracts them differently from another and
// the choice of S changes no bit of the result: S = 1 routes the maps'
// multiplies to the integer pipes (sf::mul, the same correctly rounded
// product), which frees the FP64 pipe that bounds the fused pass on GB300.
template <int S>
__device__ __forceinline__ void ensure_knl(Part& p, const MapCtx& m) {
  if (!p.knl_ok) {
    p.dp_p = dmul<S>(p.dE, m.dp_p_coeff);
    p.knl = __drcp_rn(__dadd_rn(1.0, p.dp_p));
    p.knl_ok = true;
  }
}

// drifti body (teapotbase.cc:132-139)
template <int S>
__device__ __forceinline__ void drift_body(Part& p, const MapCtx& m, double L) {
  ensure_knl<S>(p, m);
  const double dp_p = p.dp_p, knl = p.knl;
  const double kl = dmul<S>(knl, L);
  p.x = fma(kl, p.xp, p.x);
  p.y = fma(kl, p.yp, p.y);
  // phifac = (xp^2 + yp^2 + dp_p^2 / gamma^2) / 2
  const double d2g = dmul<S>(dmul<S>(dp_p, dp_p), m.gamma2i);
  double phifac = dhalf<S>(fma(p.xp, p.xp, fma(p.yp, p.yp, d2g)));
  phifac = dmul<S>(fma(phifac, knl, -dmul<S>(dp_p, m.gamma2i)), knl);
  p.z = fma(-L, phifac, p.z);
}

// multpfringeIN/OUT (teapotbase.cc:395-486, 508-599), with l = pole + 1,
// z = x + i y and kt the signed kterm (IN: -kterm, OUT: +kterm, folded in
// on the host).  The reference forms six complex products and keeps their
// real parts; their terms satisfy, exactly,
//   dxfxterm = l(l+1) conj(z),      dyfyterm = -l(l+1) conj(z),
//   dyfxterm = (l+1)((l+2) y, (l-2) x),  dxfyterm = (l+1)((l-2) y, (l+2) x),
// so with kt z^(l-1) = A + i B and kt z^l = C + i D the six real parts are
//   dxfxcx = l(l+1)(A x + B y) = -dyfycx,
//   dyfxcx = (l+1)(l+2) A y - (l+1)(l-2) B x,
//   dxfycx = (l+1)(l-2) A y - (l+1)(l+2) B x,
//   fxcx = l C x + (l+2) D y,  fycx = l C y - (l+2) D x,
// and detM = 1 - e with e = u^2 + M12 M21 (u = dxfxcx KNL), whose inverse
// is a short series for small e.  46 FP64 operations instead of ~110 and
// two divisions; the results differ from the reference's by roundings.
// c = {kt_re, kt_im, l, l+2, l(l+1), (l+1)(l+2), (l+1)(l-2)}, i0 = pole.
template <int S>
__device__ __forceinline__ void multpfringe_body(Part& p, const MapCtx& m, const DevOp& o) {
  ensure_knl<S>(p, m);
  const double x = p.x, y = p.y, px = p.xp, py = p.yp, KNL = p.knl;
  double zr = 1.0, zi = 0.0;  // z^(l-1)
  if (o.i0 > 0) {
    zr = x;
    zi = y;
    for (int q = 1; q < o.i0; ++q) {
      const double t = fma(zr, x, -dmul<S>(zi, y));
      zi = fma(zr, y, dmul<S>(zi, x));
      zr = t;
    }
  }
  const double ktr = o.c[0], kti = o.c[1];
  const double A = fma(ktr, zr, -dmul<S>(kti, zi)), B = fma(ktr, zi, dmul<S>(kti, zr));
  const double C = fma(A, x, -dmul<S>(B, y)), D = fma(A, y, dmul<S>(B, x));
  const double lC = dmul<S>(o.c[2], C), lp2D = dmul<S>(o.c[3], D);
  const double fx = fma(lC, x, dmul<S>(lp2D, y));
  const double fy = fma(lC, y, -dmul<S>(lp2D, x));
  const double dxfx = dmul<S>(o.c[4], fma(A, x, dmul<S>(B, y)));
  const double dyfx = fma(dmul<S>(o.c[5], A), y, -dmul<S>(dmul<S>(o.c[6], B), x));
  const double dxfy = fma(dmul<S>(o.c[6], A), y, -dmul<S>(dmul<S>(o.c[5], B), x));
  p.x = fma(-fx, KNL, x);
  p.y = fma(-fy, KNL, y);
  const double u = dmul<S>(dxfx, KNL);  // M11 = 1 - u, M22 = 1 + u
  const double M12 = -dmul<S>(dxfy, KNL), M21 = -dmul<S>(dyfx, KNL);
  const double e = fma(u, u, dmul<S>(M12, M21));  // detM = 1 - e
  const double nxp = fma(-M12, py, fma(u, px, px));   // M22 px - M12 py
  const double nyp = fma(-M21, px, fma(-u, py, py));  // -M21 px + M11 py
  const long long eb = __double_as_longlong(e) & 0x7FFFFFFFFFFFFFFFll;
  double pxnew, pynew;
  if (eb < 0x3E40000000000000ll) {  // |e| < 2^-27: 1/(1-e) = 1 + e + O(2^-54)
    pxnew = fma(nxp, e, nxp);
    pynew = fma(nyp, e, nyp);
  } else if (eb < 0x3EB0000000000000ll) {  // |e| < 2^-20: 1 + e + e^2
    const double w = fma(e, e, e);
    pxnew = fma(nxp, w, nxp);
    pynew = fma(nyp, w, nyp);
  } else {
    const double detM = __dsub_rn(1.0, e);
    pxnew = __ddiv_rn(nxp, detM);
    pynew = __ddiv_rn(nyp, detM);
  }
  p.xp = pxnew;
  p.yp = pynew;
  p.z = fma(-dmul<S>(fma(pxnew, fx, dmul<S>(pynew, fy)), KNL), KNL, p.z);
}

// Applies ops[a..b) to one particle.
template <int S>
__device__ __forceinline__ void apply_ops(Part& p, const DevOp* __restrict__ ops, int a, int b,
                                          const MapCtx& m) {
  // S: a bit per map family selects its multiplies' pipe (1 = integer):
  // bit 0 drift, quad2 / bend2 and the wedges; bit 1 quad1; bit 2 the quad
  // fringes; bit 3 bends, bend fringes, multipoles and their fringes,
  // rotations.  The results are the same for every S.
  constexpr int SD = S & 1, SQ = (S >> 1) & 1, SF = (S >> 2) & 1, SB = (S >> 3) & 1;
  for (int k = a; k < b; ++k) {
    const DevOp& o = ops[k];
    switch (o.code) {
      case ORBIT_OP_DRIFT:  // drift (teapotbase.cc:158-184)
        drift_body<SD>(p, m, o.c[0]);
        break;
      case ORBIT_OP_QUAD1: {  // quad1 (teapotbase.cc:620-701); c = m11,m12,m21,m22,m33,m34,m43,m44,g2i*L
        ensure_knl<SQ>(p, m);
        const double x0 = p.x, xp0 = p.xp, y0 = p.y, yp0 = p.yp;
        p.x = fma(x0, o.c[0], dmul<SQ>(xp0, o.c[1]));
        p.xp = fma(x0, o.c[2], dmul<SQ>(xp0, o.c[3]));
        p.y = fma(y0, o.c[4], dmul<SQ>(yp0, o.c[5]));
        p.yp = fma(y0, o.c[6], dmul<SQ>(yp0, o.c[7]));
        p.z = fma(p.dp_p, o.c[8], p.z);
        break;
      }
      case ORBIT_OP_QUAD2:
      case ORBIT_OP_BEND2: {  // quad2 / bend2 (teapotbase.cc:719-744, 1164-1189); c0 = L
        ensure_knl<SD>(p, m);
        const double L = o.c[0], dp_p = p.dp_p, knl = p.knl;
        const double kld = dmul<SD>(dmul<SD>(knl, L), dp_p);
        p.x = fma(-kld, p.xp, p.x);
        p.y = fma(-kld, p.yp, p.y);
        const double d2g = dmul<SD>(dmul<SD>(dp_p, dp_p), m.gamma2i);
        double phifac = dhalf<SD>(fma(p.xp, p.xp, fma(p.yp, p.yp, d2g)));
        phifac = dmul<SD>(fma(phifac, knl, d2g), knl);
        p.z = fma(-L, phifac, p.z);
        break;
      }
      case ORBIT_OP_QFRIN:
      case ORBIT_OP_QFROUT: {  // quadfringeIN/OUT (teapotbase.cc:784-904); c0 = +-kq/4, c1 = +-kq/12
        ensure_knl<SF>(p, m);
        // Regrouped for the FP64 pipe: k4 folded into r^2 and x y, the
        // products k12 x0 a and k12 y0 b shared by x, y and z, and the
        // test on u made on its bits (u >= 0) on the integer pipe.
        const double KNL = p.knl;
        const double x0 = p.x, xp0 = p.xp, y0 = p.y, yp0 = p.yp;
        const double x2 = dmul<SF>(x0, x0), y2 = dmul<SF>(y0, y0);
        const double k4 = dmul<SF>(o.c[0], KNL), k12 = dmul<SF>(o.c[1], KNL);
        const double a = fma(3., y2, x2), b = fma(3., x2, y2);  // x^2+3y^2, y^2+3x^2
        const double t = dmul<SF>(k4, __dsub_rn(x2, y2));
        const double u = dmul<SF>(t, t);  // detM = 1 - u
        const double kr = dmul<SF>(k4, __dadd_rn(x2, y2)), kxy = dmul<SF>(dtwice<SF>(k4), dmul<SF>(x0, y0));
        const double nxp = fma(kxy, yp0, fma(-kr, xp0, xp0));  // xp0 - k4 (xp0 r^2 - 2 yp0 x y)
        const double nyp = fma(-kxy, xp0, fma(kr, yp0, yp0));  // yp0 - k4 (-yp0 r^2 + 2 xp0 x y)
        const long long ub = __double_as_longlong(u);
        if (ub < 0x3E40000000000000ll) {
          // u < 2^-27: 1/(1-u) = 1 + u + O(2^-54)
          p.xp = fma(nxp, u, nxp);
          p.yp = fma(nyp, u, nyp);
        } else if (ub < 0x3EB0000000000000ll) {
          // u < 2^-20: 1/(1-u) = 1 + u + u^2 + O(2^-60)
          const double w = fma(u, u, u);
          p.xp = fma(nxp, w, nxp);
          p.yp = fma(nyp, w, nyp);
        } else {
          const double detM = __dsub_rn(1.0, u);
          p.xp = __ddiv_rn(nxp, detM);
          p.yp = __ddiv_rn(nyp, detM);
        }
        const double X = dmul<SF>(dmul<SF>(k12, x0), a), Y = dmul<SF>(dmul<SF>(k12, y0), b);
        p.x = __dadd_rn(x0, X);
        p.y = __dsub_rn(y0, Y);
        p.z = fma(KNL, fma(xp0, X, -dmul<SF>(yp0, Y)), p.z);
        break;
      }
      case ORBIT_OP_BEND1: {  // bend1 (teapotbase.cc:1099-1146); c = m11,m12,m16,m21,m22,m26,m51,m52,m56,L
        ensure_knl<SB>(p, m);
        const double x0 = p.x, xp0 = p.xp, dp_p = p.dp_p;
        p.x = fma(x0, o.c[0], fma(xp0, o.c[1], dmul<SB>(dp_p, o.c[2])));
        p.xp = fma(x0, o.c[3], fma(xp0, o.c[4], dmul<SB>(dp_p, o.c[5])));
        p.y = fma(o.c[9], p.yp, p.y);
        p.z = __dadd_rn(p.z, fma(x0, o.c[6], fma(xp0, o.c[7], dmul<SB>(dp_p, o.c[8]))));
        break;
      }
      case ORBIT_OP_BEND3: {  // bend3 (teapotbase.cc:1208-1232); c0 = th
        ensure_knl<SB>(p, m);
        const double th = o.c[0], dp_p = p.dp_p, KNL = p.knl;
        double phifac = dhalf<SB>(fma(p.yp, p.yp, dmul<SB>(dmul<SB>(dp_p, dp_p), m.gamma2i)));
        p.xp = fma(-dmul<SB>(phifac, KNL), th, p.xp);
        p.y = fma(dmul<SB>(dmul<SB>(KNL, p.yp), p.x), th, p.y);
        phifac = dmul<SB>(fma(phifac, KNL, -dmul<SB>(dp_p, m.gamma2i)), KNL);
        p.z = fma(-dmul<SB>(th, phifac), p.x, p.z);
        break;
      }
      case ORBIT_OP_BEND4: {  // bend4 (teapotbase.cc:1251-1274); c0 = th
        ensure_knl<SB>(p, m);
        const double th = o.c[0], KNL = p.knl;
        const double xfac = fma(dhalf<SB>(dmul<SB>(KNL, p.xp)), th, 1.0);
        const double kxp = dmul<SB>(KNL, p.xp);
        const double phifac = dhalf<SB>(dmul<SB>(kxp, kxp));
        p.x = dmul<SB>(p.x, dmul<SB>(xfac, xfac));
        p.xp = __ddiv_rn(p.xp, xfac);
        p.z = fma(-dmul<SB>(th, phifac), p.x, p.z);
        break;
      }
      case ORBIT_OP_BFRIN:
      case ORBIT_OP_BFROUT: {  // bendfringeIN/OUT (teapotbase.cc:1292-1348); c0 = +-1/(2 rho), c1 = +-1/rho
        ensure_knl<SB>(p, m);
        const double KNL = p.knl, y2 = dmul<SB>(p.y, p.y), xp0 = p.xp;
        p.x = fma(dmul<SB>(KNL, y2), o.c[0], p.x);
        p.yp = fma(-dmul<SB>(dmul<SB>(KNL, xp0), p.y), o.c[1], p.yp);
        p.z = fma(dmul<SB>(dmul<SB>(dmul<SB>(KNL, KNL), xp0), y2), o.c[0], p.z);
        break;
      }
      case ORBIT_OP_MULTP: {  // multp (teapotbase.cc:336-374); i0 = pole, i1 = skew, c0 = kl/pole!
        if (m.charge == 0.) break;
        // z^pole from z (the reference starts its loop from 1), kl/pole! on
        // the host
        double zr = 1.0, zi = 0.0;
        if (o.i0 > 0) {
          zr = p.x;
          zi = p.y;
          for (int q = 1; q < o.i0; ++q) {
            const double t = fma(zr, p.x, -dmul<SB>(zi, p.y));
            zi = fma(zr, p.y, dmul<SB>(zi, p.x));
            zr = t;
          }
        }
        const double kl1 = o.c[0];
        if (o.i1) {
          p.xp = fma(kl1, zi, p.xp);
          p.yp = fma(kl1, zr, p.yp);
        } else {
          p.xp = fma(-kl1, zr, p.xp);
          p.yp = fma(kl1, zi, p.yp);
        }
        break;
      }
      case ORBIT_OP_MPFRIN:
      case ORBIT_OP_MPFROUT:  // c0, c1 = signed kterm (re, im)
        if (m.charge == 0.) break;
        multpfringe_body<SB>(p, m, o);
        break;
      case ORBIT_OP_ROTXY: {  // rotatexy (teapotbase.cc:80-101); c0 = cos, c1 = sin
        const double cs = o.c[0], sn = o.c[1];
        const double xt = p.x, pxt = p.xp, yt = p.y, pyt = p.yp;
        p.x = fma(cs, xt, -dmul<SB>(sn, yt));
        p.xp = fma(cs, pxt, -dmul<SB>(sn, pyt));
        p.y = fma(sn, xt, dmul<SB>(cs, yt));
        p.yp = fma(sn, pxt, dmul<SB>(cs, pyt));
        break;
      }
      case ORBIT_OP_WRAP:  // wrapbunch (teapotbase.cc:202-212); c0 = L, c1 = L/2
        if (p.z < -o.c[1]) p.z = __dadd_rn(p.z, o.c[0]);
        if (p.z > o.c[1]) p.z = __dsub_rn(p.z, o.c[0]);
        break;
      case ORBIT_OP_KICK:  // kick (teapotbase.cc:232-258)
        if (o.c[0] != 0.) p.xp = __dadd_rn(p.xp, o.c[0]);
        if (o.c[1] != 0.) p.yp = __dadd_rn(p.yp, o.c[1]);
        if (o.c[2] != 0.) { p.dE = __dadd_rn(p.dE, o.c[2]); p.knl_ok = false; }
        break;
      case ORBIT_OP_WEDGEROT: {  // wedgerotate (teapotbase.cc:923-967); c0 = cos, c1 = sin, i0 = frinout
        // dE = (p0 - 1)/coeff cancels, so this rare map keeps the
        // reference's unfused rounding (explicit _rn operations).
        const double cs = o.c[0], sn = o.c[1];
        const double dpc = m.dp_p_coeff;
        double dp_p;
        if (o.i0 == 0) {
          dp_p = __dmul_rn(p.dE, dpc);
          const double xp_t = p.xp, p0_t = __dadd_rn(1.0, dp_p);
          p.x = __ddiv_rn(p.x, cs);
          p.xp = __dadd_rn(__dmul_rn(xp_t, cs), __dmul_rn(p0_t, sn));
          const double p0 = __dadd_rn(__dmul_rn(-xp_t, sn), __dmul_rn(p0_t, cs));
          dp_p = __dsub_rn(p0, 1.0);
          p.z = __dmul_rn(__dadd_rn(__dmul_rn(-p.x, sn), p.z), cs);
        } else {
          dp_p = __dmul_rn(p.dE, dpc);
          const double p0 = __dadd_rn(1.0, dp_p);
          p.z = __dadd_rn(__dmul_rn(p.x, sn), __ddiv_rn(p.z, cs));
          p.x = __dmul_rn(p.x, cs);
          const double xp_t = __dsub_rn(__dmul_rn(p.xp, cs), __dmul_rn(p0, sn));
          const double p0_t = __dadd_rn(__dmul_rn(p.xp, sn), __dmul_rn(p0, cs));
          p.xp = xp_t;
          dp_p = __dsub_rn(p0_t, 1.0);
        }
        p.dE = __ddiv_rn(dp_p, dpc);
        p.knl_ok = false;
        break;
      }
      case ORBIT_OP_WEDGEDRIFT: {  // wedgedrift (teapotbase.cc:986-1016); c0 = ct, i0 = inout
        double s;
        if (o.i0 == 0) {
          ensure_knl<SD>(p, m);
          const double tn = __ddiv_rn(p.xp, __dadd_rn(1.0, p.dp_p));
          s = __ddiv_rn(p.x, __dsub_rn(o.c[0], tn));
        } else {
          s = __ddiv_rn(p.x, o.c[0]);
        }
        drift_body<SD>(p, m, s);
        break;
      }
      case ORBIT_OP_WEDGEBEND: {  // wedgebend (teapotbase.cc:1037-1080); c0 = ct, c1 = rho, i0 = inout, i1 = nst
        double s;
        if (o.i0 == 0) {
          s = __ddiv_rn(-p.x, o.c[0]);
        } else {
          ensure_knl<SD>(p, m);
          const double tn = __ddiv_rn(p.xp, __dadd_rn(1.0, p.dp_p));
          s = __ddiv_rn(-p.x, __dadd_rn(o.c[0], tn));
        }
        const int nst = o.i1;
        const double sm = __ddiv_rn(s, (double)nst), sm2 = __ddiv_rn(sm, 2.0);
        const double kick = __ddiv_rn(sm, o.c[1]);
        drift_body<SD>(p, m, sm2);
        p.xp = __dsub_rn(p.xp, kick);
        for (int j = 1; j < nst; j++) {
          drift_body<SD>(p, m, sm);
          p.xp = __dsub_rn(p.xp, kick);
        }
        drift_body<SD>(p, m, sm2);
        break;
      }
      default:
        break;
    }
  }
}

// Host: compiles a reference op into a DevOp with the per-element constants
// computed as the reference computes them; returns false for an unknown code.
// `time_adv` receives length/v for maps that advance SyncPart time, or 0.
bool compile_op(const orbit_op_t& in, const orbit_sync_t& s, DevOp& out, double* time_adv);
MapCtx make_ctx(const orbit_sync_t& s);

}  // namespace orbit
