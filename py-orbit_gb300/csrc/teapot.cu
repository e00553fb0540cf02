// Host-side op compilation and the single-map kernels behind the
// orbit_tpb_* entry points (src/teapot/wrap_teapotbase.cc:488-512).
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "teapot.cuh"

namespace orbit {

static const double kC = 2.99792458e+8;  // OrbitConst.cc:27

static double factorial(int n) {  // teapotbase.cc:45-57
  double f = 1.0;
  for (int i = 1; i <= n; ++i) f = i * f;
  return f;
}

MapCtx make_ctx(const orbit_sync_t& s) {
  MapCtx m;
  m.dp_p_coeff = 1.0 / (s.momentum * s.beta);
  m.gamma2i = 1.0 / (s.gamma * s.gamma);
  m.charge = s.charge;
  return m;
}

bool compile_op(const orbit_op_t& in, const orbit_sync_t& s, DevOp& o, double* time_adv) {
  std::memset(&o, 0, sizeof(o));
  o.code = in.code;
  o.i0 = in.i0;
  o.i1 = in.i1;
  o.i2 = in.i2;
  double v = kC * s.beta;
  *time_adv = 0.0;
  const double* d = in.d;
  switch (in.code) {
    case ORBIT_OP_DRIFT:
      o.c[0] = d[0];
      *time_adv = d[0] / v;
      return true;
    case ORBIT_OP_QUAD1: {
      double length = d[0], kqc = d[1];
      if (kqc == 0. || s.charge == 0.) {  // teapotbase.cc:622-626
        o.code = ORBIT_OP_DRIFT;
        o.c[0] = length;
        *time_adv = length / v;
        return true;
      }
      if (length > 0.) *time_adv = length / v;
      double sq, kl, cx, sx, cy, sy;
      double m11, m12, m21, m22, m33, m34, m43, m44;
      if (kqc > 0.) {  // teapotbase.cc:647-663
        sq = std::pow(kqc, 0.5);
        kl = sq * length;
        cx = std::cos(kl); sx = std::sin(kl); cy = std::cosh(kl); sy = std::sinh(kl);
        m11 = cx; m12 = sx / sq; m21 = -sx * sq; m22 = cx;
        m33 = cy; m34 = sy / sq; m43 = sy * sq; m44 = cy;
      } else {  // teapotbase.cc:664-680
        sq = std::pow(-kqc, 0.5);
        kl = sq * length;
        cx = std::cosh(kl); sx = std::sinh(kl); cy = std::cos(kl); sy = std::sin(kl);
        m11 = cx; m12 = sx / sq; m21 = sx * sq; m22 = cx;
        m33 = cy; m34 = sy / sq; m43 = -sy * sq; m44 = cy;
      }
      double g2i = 1.0 / (s.gamma * s.gamma);
      o.c[0] = m11; o.c[1] = m12; o.c[2] = m21; o.c[3] = m22;
      o.c[4] = m33; o.c[5] = m34; o.c[6] = m43; o.c[7] = m44;
      o.c[8] = g2i * length;
      return true;
    }
    case ORBIT_OP_QUAD2:
    case ORBIT_OP_BEND2:
      o.c[0] = d[0];
      return true;
    case ORBIT_OP_QFRIN:
    case ORBIT_OP_QFROUT:
      if (s.charge == 0.) { o.code = 0; return true; }
      {
        // the OUT map is the IN map with kq -> -kq (teapotbase.cc:784-904);
        // both factors scale exactly under the sign flip
        double sg = (in.code == ORBIT_OP_QFRIN) ? 1.0 : -1.0;
        o.c[0] = sg * (d[0] / 4.);
        o.c[1] = sg * (d[0] / 12.);
      }
      return true;
    case ORBIT_OP_BEND1: {  // teapotbase.cc:1099-1131
      double length = d[0], th = d[1];
      if (length > 0.) *time_adv = length / v;
      double betasq = s.beta * s.beta;
      double rho = length / th, cx = std::cos(th), sx = std::sin(th);
      o.c[0] = cx; o.c[1] = rho * sx; o.c[2] = rho * (1.0 - cx);
      o.c[3] = -sx / rho; o.c[4] = cx; o.c[5] = sx;
      o.c[6] = -sx; o.c[7] = -rho * (1.0 - cx); o.c[8] = -betasq * length + rho * sx;
      o.c[9] = length;
      return true;
    }
    case ORBIT_OP_BEND3:
    case ORBIT_OP_BEND4:
      o.c[0] = d[0];
      return true;
    case ORBIT_OP_BFRIN:
    case ORBIT_OP_BFROUT: {
      double sg = (in.code == ORBIT_OP_BFRIN) ? 1.0 : -1.0;
      o.c[0] = sg / (2. * d[0]);
      o.c[1] = sg / d[0];
      return true;
    }
    case ORBIT_OP_MULTP:
      if (in.i0 < 0 || in.i0 > 45) return false;
      o.c[0] = d[0] / factorial(in.i0);  // teapotbase.cc:349
      return true;
    case ORBIT_OP_MPFRIN:
    case ORBIT_OP_MPFROUT: {
      if (in.i0 < 0 || in.i0 > 45) return false;
      double kf = d[0] / (4.0 * factorial(in.i0 + 2));  // teapotbase.cc:417
      double sg = (in.code == ORBIT_OP_MPFRIN) ? -1.0 : 1.0;
      if (in.i1) { o.c[0] = 0.0 * sg; o.c[1] = sg * kf; }
      else { o.c[0] = sg * kf; o.c[1] = 0.0 * sg; }
      double l = (double)(in.i0 + 1);  // the integer factors of the regrouped terms
      o.c[2] = l;
      o.c[3] = l + 2.0;
      o.c[4] = l * (l + 1.0);
      o.c[5] = (l + 1.0) * (l + 2.0);
      o.c[6] = (l + 1.0) * (l - 2.0);
      return true;
    }
    case ORBIT_OP_ROTXY:
      o.c[0] = std::cos(d[0]);
      o.c[1] = std::sin(d[0]);
      return true;
    case ORBIT_OP_WRAP:
      o.c[0] = d[0];
      o.c[1] = d[0] / 2.0;
      return true;
    case ORBIT_OP_KICK:
      o.c[0] = d[0]; o.c[1] = d[1]; o.c[2] = d[2];
      return true;
    case ORBIT_OP_WEDGEROT:
      o.c[0] = std::cos(d[0]);
      o.c[1] = std::sin(d[0]);
      return true;
    case ORBIT_OP_WEDGEDRIFT:
      o.c[0] = std::cos(d[0]) / std::sin(d[0]);
      return true;
    case ORBIT_OP_WEDGEBEND: {
      o.c[0] = std::cos(d[0]) / std::sin(d[0]);
      o.c[1] = d[1];
      int nst = in.i1 / 2;
      if (nst < 1) nst = 1;
      o.i1 = nst;
      return true;
    }
    default:
      return false;
  }
}

// One map over all particles: the eager path of the orbit_tpb_* calls.
__global__ void __launch_bounds__(256) k_apply_one(double* __restrict__ cx, double* __restrict__ cxp,
                                                   double* __restrict__ cy, double* __restrict__ cyp,
                                                   double* __restrict__ cz, double* __restrict__ cdE,
                                                   int n, DevOp op, MapCtx m) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    Part p;
    p.x = cx[i]; p.xp = cxp[i]; p.y = cy[i]; p.yp = cyp[i]; p.z = cz[i]; p.dE = cdE[i];
    p.knl_ok = false;
    apply_ops<ORBIT_SOFT_MUL>(p, &op, 0, 1, m);
    cx[i] = p.x; cxp[i] = p.xp; cy[i] = p.y; cyp[i] = p.yp; cz[i] = p.z; cdE[i] = p.dE;
  }
}

// teapot_base function names (src/teapot/wrap_teapotbase.cc:488-512) by op code.
static const char* tpb_name(int code) {
  switch (code) {
    case ORBIT_OP_DRIFT: return "teapot_base.drift";
    case ORBIT_OP_QUAD1: return "teapot_base.quad1";
    case ORBIT_OP_QUAD2: return "teapot_base.quad2";
    case ORBIT_OP_QFRIN: return "teapot_base.quadfringeIN";
    case ORBIT_OP_QFROUT: return "teapot_base.quadfringeOUT";
    case ORBIT_OP_BEND1: return "teapot_base.bend1";
    case ORBIT_OP_BEND2: return "teapot_base.bend2";
    case ORBIT_OP_BEND3: return "teapot_base.bend3";
    case ORBIT_OP_BEND4: return "teapot_base.bend4";
    case ORBIT_OP_BFRIN: return "teapot_base.bendfringeIN";
    case ORBIT_OP_BFROUT: return "teapot_base.bendfringeOUT";
    case ORBIT_OP_MULTP: return "teapot_base.multp";
    case ORBIT_OP_MPFRIN: return "teapot_base.multpfringeIN";
    case ORBIT_OP_MPFROUT: return "teapot_base.multpfringeOUT";
    case ORBIT_OP_ROTXY: return "teapot_base.rotatexy";
    case ORBIT_OP_WRAP: return "teapot_base.wrapbunch";
    case ORBIT_OP_KICK: return "teapot_base.kick";
    case ORBIT_OP_WEDGEROT: return "teapot_base.wedgerotate";
    case ORBIT_OP_WEDGEDRIFT: return "teapot_base.wedgedrift";
    case ORBIT_OP_WEDGEBEND: return "teapot_base.wedgebend";
    default: return "teapot_base";
  }
}

static int launch_one(orbit_bunch_t* b, const orbit_op_t& op) {
  ORBIT_NVTX(tpb_name(op.code));
  if (!b) return set_error(ORBIT_ERR_ARG, "null bunch");
  DevOp d;
  double tadv = 0.0;
  if (!compile_op(op, b->sync, d, &tadv)) return set_error(ORBIT_ERR_ARG, "bad map parameters");
  b->sync.time = b->sync.time + tadv;  // SyncPart::setTime (teapotbase.cc:165)
  if (b->n == 0 || d.code == 0) return ORBIT_OK;
  int threads = 256;
  int blocks = (b->n + threads - 1) / threads;
  int cap = num_sms() * 8;
  if (blocks > cap) blocks = cap;
  k_apply_one<<<blocks, threads, 0, b->stream>>>(b->coord(0), b->coord(1), b->coord(2), b->coord(3),
                                                  b->coord(4), b->coord(5), b->n, d, make_ctx(b->sync));
  ORBIT_LAUNCH_CHECK("k_apply_one");
  return ORBIT_OK;
}

static orbit_op_t mk(int code, double d0 = 0, double d1 = 0, double d2 = 0, int i0 = 0, int i1 = 0) {
  orbit_op_t o;
  std::memset(&o, 0, sizeof(o));
  o.code = code;
  o.d[0] = d0; o.d[1] = d1; o.d[2] = d2;
  o.i0 = i0; o.i1 = i1;
  return o;
}

}  // namespace orbit

using namespace orbit;

extern "C" {
int orbit_tpb_rotatexy(orbit_bunch_t* b, double a) { return launch_one(b, mk(ORBIT_OP_ROTXY, a)); }
int orbit_tpb_drift(orbit_bunch_t* b, double L) { return launch_one(b, mk(ORBIT_OP_DRIFT, L)); }
int orbit_tpb_wrapbunch(orbit_bunch_t* b, double L) { return launch_one(b, mk(ORBIT_OP_WRAP, L)); }
int orbit_tpb_kick(orbit_bunch_t* b, double kx, double ky, double kE) { return launch_one(b, mk(ORBIT_OP_KICK, kx, ky, kE)); }
int orbit_tpb_multp(orbit_bunch_t* b, int pole, double kl, int skew) { return launch_one(b, mk(ORBIT_OP_MULTP, kl, 0, 0, pole, skew)); }
int orbit_tpb_multpfringeIN(orbit_bunch_t* b, int pole, double kl, int skew) { return launch_one(b, mk(ORBIT_OP_MPFRIN, kl, 0, 0, pole, skew)); }
int orbit_tpb_multpfringeOUT(orbit_bunch_t* b, int pole, double kl, int skew) { return launch_one(b, mk(ORBIT_OP_MPFROUT, kl, 0, 0, pole, skew)); }
int orbit_tpb_quad1(orbit_bunch_t* b, double L, double kq) { return launch_one(b, mk(ORBIT_OP_QUAD1, L, kq)); }
int orbit_tpb_quad2(orbit_bunch_t* b, double L) { return launch_one(b, mk(ORBIT_OP_QUAD2, L)); }
int orbit_tpb_quadfringeIN(orbit_bunch_t* b, double kq) { return launch_one(b, mk(ORBIT_OP_QFRIN, kq)); }
int orbit_tpb_quadfringeOUT(orbit_bunch_t* b, double kq) { return launch_one(b, mk(ORBIT_OP_QFROUT, kq)); }
int orbit_tpb_wedgerotate(orbit_bunch_t* b, double e, int fr) { return launch_one(b, mk(ORBIT_OP_WEDGEROT, e, 0, 0, fr)); }
int orbit_tpb_wedgedrift(orbit_bunch_t* b, double e, int io) { return launch_one(b, mk(ORBIT_OP_WEDGEDRIFT, e, 0, 0, io)); }
int orbit_tpb_wedgebend(orbit_bunch_t* b, double e, int io, double rho, int ns) { return launch_one(b, mk(ORBIT_OP_WEDGEBEND, e, rho, 0, io, ns)); }
int orbit_tpb_bend1(orbit_bunch_t* b, double L, double th) { return launch_one(b, mk(ORBIT_OP_BEND1, L, th)); }
int orbit_tpb_bend2(orbit_bunch_t* b, double L) { return launch_one(b, mk(ORBIT_OP_BEND2, L)); }
int orbit_tpb_bend3(orbit_bunch_t* b, double th) { return launch_one(b, mk(ORBIT_OP_BEND3, th)); }
int orbit_tpb_bend4(orbit_bunch_t* b, double th) { return launch_one(b, mk(ORBIT_OP_BEND4, th)); }
int orbit_tpb_bendfringeIN(orbit_bunch_t* b, double rho) { return launch_one(b, mk(ORBIT_OP_BFRIN, rho)); }
int orbit_tpb_bendfringeOUT(orbit_bunch_t* b, double rho) { return launch_one(b, mk(ORBIT_OP_BFROUT, rho)); }
}
