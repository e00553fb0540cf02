// Lattice programs: a recorded node sequence (the order AccNode.trackActions
// produces, py/orbit/lattice/AccNode.py:302-350) compiled into fused device
// passes and replayed from a CUDA graph.
//
// A turn with SC kicks S_0..S_{m-1} between map segments M_0..M_m runs as
//   [P_0]  solve(S_0) P_1 solve(S_1) ... solve(S_{m-1}) P_m
// where P_0 = M_0 + extrema(S_0), P_i = kick(S_{i-1}) + M_i + extrema(S_i) and
// the last pass of a turn that is followed by another turn also applies M_0
// of the next turn and the extrema scan for its first kick.  Every pass reads
// and writes the six coordinates once; the deposit reads x, y, z once more.
#include <cstring>
#include <vector>

#include "common.cuh"
#include "sc2p5d.cuh"
#include "sc_device.cuh"
#include "teapot.cuh"
#include "batch.cuh"
#include "program.cuh"

namespace orbit {

static const int kPassSmem = 220 * 1024;

// Threads per block of the fused pass (one block per SM when the kick keeps
// its potential in shared memory); the register budget per thread is
// 65536 / ORBIT_PASS_THREADS.
#ifndef ORBIT_PASS_THREADS
#define ORBIT_PASS_THREADS 512
#endif

// Copies n elements of global memory (written by an earlier kernel) into
// shared memory with asynchronous 16-byte copies (cp.async.cg: no
// registers held, every copy of the thread in flight at once), then applies
// f in place to the elements this thread copied, once they have landed
// (cp.async.wait_all waits for the thread's own copies).  Threads t0.. of
// the block take part.  Where either address is not 16-byte aligned the
// thread copies element by element instead.  Returns with this thread's
// elements final; the caller synchronises the block.
template <typename T, typename F>
__device__ __forceinline__ void copy_smem_async(T* s, const T* g, int n, F f, int t0) {
  const int t = (int)threadIdx.x - t0, nt = (int)blockDim.x - t0;
  if (t < 0) return;
  constexpr int E = 16 / (int)sizeof(T);  // elements per 16-byte copy
  const uint32_t sb = (uint32_t)__cvta_generic_to_shared(s);
  const bool aligned = ((sb | (uint32_t)(size_t)g) & 15u) == 0u;
  const int nb = aligned ? n / E : 0;
  for (int i = t; i < nb; i += nt)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sb + 16u * (uint32_t)i),
                 "l"(reinterpret_cast<const char*>(g) + 16 * (size_t)i)
                 : "memory");
  asm volatile("cp.async.commit_group;" ::: "memory");
  asm volatile("cp.async.wait_all;" ::: "memory");
  for (int i = t; i < nb; i += nt) {
#pragma unroll
    for (int q = 0; q < E; ++q) s[i * E + q] = f(s[i * E + q]);
  }
  for (int i = nb * E + t; i < n; i += nt) s[i] = f(__ldcg(g + i));
}

// The kick constants of a pass (one thread), out of line so that their
// registers do not weigh on the particle loop's.
__device__ __noinline__ void kick_consts_into(KickConst* k, KickFix* kf, const KickArgs& kick) {
  load_kick_const(*k, kick.st, kick.host_factor, kick.nx, kick.ny, kick.nz, kf == nullptr);
  if (kf) load_kick_fix(*kf, kick.st, k->fac, kick.nx, kick.ny, kick.nz);
}

// KF: 0 no kick, 1 plain kick, 2 fp32 kick.  EXT: accumulate extrema.
// Blocks blk = 0..nblk-1 share the bunch's particles.
template <int KF, bool EXT, bool KSMEM>
__device__ __forceinline__ void pass_body(double* __restrict__ cx, double* __restrict__ cxp,
                                          double* __restrict__ cy, double* __restrict__ cyp,
                                          double* __restrict__ cz, double* __restrict__ cdE, int n,
                                          const DevOp* __restrict__ ops, int a, int b, const MapCtx& m,
                                          const KickArgs& kick, ScState* ext_st, unsigned* status,
                                          const SetupArgs& sa, double* __restrict__ knl_buf, int km, int blk,
                                          int nblk) {
  KickConst k;
  KickFix kf;
  const long long* P = kick.phi_fix;
  const long long* Lm = kick.lam_fix;
  const float* Pf = kick.phi_f;
  const float* Lf = kick.lam_f;
  extern __shared__ __align__(16) unsigned char s_raw[];
  if (KF != 0) {
    // thread 0 computes the kick constants (two FP64 divisions among
    // them) while warps 1.. fill the block's copy of the potential and the
    // line density; one barrier completes both
    __shared__ KickConst s_k;
    __shared__ KickFix s_kf;
    if (threadIdx.x == 0) kick_consts_into(&s_k, KF == 1 ? &s_kf : nullptr, kick);
    if (KSMEM) {
      const int ng = kick.nx * kick.ny, t0 = blockDim.x > 64 ? 32 : 0;
      if (KF == 1) {
        // fixed-point copy converted here from the FP64 potential, at the
        // scales the kick constants use
        const int sphi = scale_bits(kick.st->phi_absmax), slam = scale_bits(kick.st->lam_absmax);
        long long* s = reinterpret_cast<long long*>(s_raw);
        // the FP64 values land in place and become 64-bit integers there
        double* sd = reinterpret_cast<double*>(s_raw);
        copy_smem_async(sd, kick.phi, ng,
                        [sphi](double v) { return __longlong_as_double(phi_fixed(v, sphi)); }, t0);
        copy_smem_async(sd + ng, kick.lam, kick.nz,
                        [slam](double v) { return __longlong_as_double(phi_fixed(v, slam)); }, t0);
        P = s;
        Lm = s + ng;
      } else {
        float* s = reinterpret_cast<float*>(s_raw);
        copy_smem_async(s, kick.phi_f, ng, [](float v) { return v; }, t0);
        copy_smem_async(s + ng, kick.lam_f, kick.nz, [](float v) { return v; }, t0);
        Pf = s;
        Lf = s + ng;
      }
    }
    __syncthreads();
    k = s_k;
    if (KF == 1) kf = s_kf;
  }
  ExtAcc acc;
  if (EXT) acc.init();
  for (int i = blk * blockDim.x + threadIdx.x; i < n; i += nblk * blockDim.x) {
    Part p;
    p.x = cx[i]; p.xp = cxp[i]; p.y = cy[i]; p.yp = cyp[i]; p.z = cz[i]; p.dE = cdE[i];
    p.knl_ok = false;
    if (km & KNL_LOAD) {  // 1/(1+dp_p) as an earlier pass of this run computed it from the same dE
      p.dp_p = dmul<ORBIT_SOFT_MUL & 1>(p.dE, m.dp_p_coeff);
      p.knl = knl_buf[i];
      p.knl_ok = true;
    }
    if (KF == 1 && !k.skip && bnd_inside(kick.bnd, p.x, p.y)) {
      if (!kick_fixed(kf, P, Lm, p.x, p.y, p.z, p.xp, p.yp))
        kick_plain(k, kick.phi, kick.lam, p.x, p.y, p.z, p.xp, p.yp);
      if (kick.lamd) {  // 2.5Drb: longitudinal kick; dE changed
        RbConst r;
        load_rb_const(r, kick.st, kick.rb_lsf);
        kick_rb_long(k, r, kick.lamd, p.x, p.y, p.z, p.dE);
        p.knl_ok = false;
      }
    }
    if (KF == 2 && !k.skip && bnd_inside(kick.bnd, p.x, p.y)) kick_fp32(k, Pf, Lf, p.x, p.y, p.z, p.xp, p.yp);
    apply_ops<ORBIT_SOFT_MUL>(p, ops, a, b, m);
    if (EXT) acc.add(p.x, p.y, p.z);
    if (km & KNL_STORE) {
      ensure_knl<ORBIT_SOFT_MUL & 1>(p, m);
      knl_buf[i] = p.knl;
    }
    cx[i] = p.x; cxp[i] = p.xp; cy[i] = p.y; cyp[i] = p.yp; cz[i] = p.z; cdE[i] = p.dE;
  }
  // the last block sets up the grids of the next kick
  if (EXT) ext_commit_and_setup(acc, ext_st, status, sa, nblk);
}

template <int KF, bool EXT, bool KSMEM>
__global__ void __launch_bounds__(ORBIT_PASS_THREADS) k_pass(double* __restrict__ cx, double* __restrict__ cxp,
                                              double* __restrict__ cy, double* __restrict__ cyp,
                                              double* __restrict__ cz, double* __restrict__ cdE, int n,
                                              const DevOp* __restrict__ ops, int a, int b, MapCtx m,
                                              KickArgs kick, ScState* ext_st, unsigned* status, SetupArgs sa,
                                              double* __restrict__ knl_buf, int km) {
  pass_body<KF, EXT, KSMEM>(cx, cxp, cy, cyp, cz, cdE, n, ops, a, b, m, kick, ext_st, status, sa, knl_buf, km,
                            blockIdx.x, gridDim.x);
}

// The same pass for the members of a batch class; each block finds its
// member in the block table.
template <int KF, bool EXT, bool KSMEM>
__global__ void __launch_bounds__(ORBIT_PASS_THREADS) kb_pass(const PassJob* __restrict__ jobs,
                                               const unsigned short* __restrict__ blk_job,
                                               const int2* __restrict__ mblk, int a, int b, int km) {
  const int j = blk_job[blockIdx.x];
  const PassJob& J = jobs[j];
  const int2 mb = mblk[j];
  pass_body<KF, EXT, KSMEM>(J.c[0], J.c[1], J.c[2], J.c[3], J.c[4], J.c[5], J.n, J.ops, a, b, J.m, J.ka, J.ext,
                            J.status, J.sa, J.knl, km, blockIdx.x - mb.x, mb.y);
}

// Shared-memory limits are raised once, outside any stream capture.
static int init_pass_attrs() {
  static bool done = false;
  if (done) return ORBIT_OK;
  ORBIT_CUDA(cudaFuncSetAttribute(k_pass<1, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kPassSmem));
  ORBIT_CUDA(cudaFuncSetAttribute(k_pass<1, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kPassSmem));
  ORBIT_CUDA(cudaFuncSetAttribute(k_pass<2, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kPassSmem));
  ORBIT_CUDA(cudaFuncSetAttribute(k_pass<2, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kPassSmem));
  ORBIT_CUDA(cudaFuncSetAttribute(kb_pass<1, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kPassSmem));
  ORBIT_CUDA(cudaFuncSetAttribute(kb_pass<1, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kPassSmem));
  done = true;
  return ORBIT_OK;
}

template <int KF, bool EXT, bool KSMEM>
static int launch_pass(orbit_bunch_t* bu, cudaStream_t s, size_t smem, const DevOp* ops, int a, int b,
                       const MapCtx& m, const KickArgs& ka, ScState* ext, const SetupArgs& sa, double* knl_buf,
                       int km) {
  int threads = ORBIT_PASS_THREADS;
  int bps = KSMEM ? (int)(kPassSmem / (smem > 0 ? smem : 1)) : 4;
  if (bps < 1) bps = 1;
  if (bps > 4) bps = 4;
  int blocks = num_sms() * bps;
  int need = (bu->n + threads - 1) / threads;
  if (need < blocks) blocks = need < 1 ? 1 : need;
  ORBIT_PB(KF == 0 ? "pass_maps" : "pass_kick_maps", s);
  k_pass<KF, EXT, KSMEM><<<blocks, threads, KSMEM ? smem : 0, s>>>(
      bu->coord(0), bu->coord(1), bu->coord(2), bu->coord(3), bu->coord(4), bu->coord(5), bu->n, ops, a, b, m, ka,
      ext, bu->d_status, sa, knl_buf, km);
  ORBIT_PE(s);
  ORBIT_LAUNCH_CHECK("k_pass");
  return ORBIT_OK;
}

size_t batch_pass_smem_limit() { return kPassSmem; }

int batch_enqueue_pass(const PassJob* jobs, const BlockMap& bm, int threads, int kf, bool ext, bool ksmem,
                       size_t smem, int a, int b, int km, cudaStream_t s, const char* tag) {
  int arc = init_pass_attrs();
  if (arc) return arc;
  const int nb = bm.nblk;
  ORBIT_PB(kf == 0 ? "batch_pass_maps" : tag, s);
  if (kf == 0) {
    if (ext) kb_pass<0, true, false><<<nb, threads, 0, s>>>(jobs, bm.blk_job, bm.mblk, a, b, km);
    else kb_pass<0, false, false><<<nb, threads, 0, s>>>(jobs, bm.blk_job, bm.mblk, a, b, km);
  } else if (ksmem) {
    if (ext) kb_pass<1, true, true><<<nb, threads, smem, s>>>(jobs, bm.blk_job, bm.mblk, a, b, km);
    else kb_pass<1, false, true><<<nb, threads, smem, s>>>(jobs, bm.blk_job, bm.mblk, a, b, km);
  } else {
    if (ext) kb_pass<1, true, false><<<nb, threads, 0, s>>>(jobs, bm.blk_job, bm.mblk, a, b, km);
    else kb_pass<1, false, false><<<nb, threads, 0, s>>>(jobs, bm.blk_job, bm.mblk, a, b, km);
  }
  ORBIT_PE(s);
  ORBIT_LAUNCH_CHECK("batch pass");
  return ORBIT_OK;
}

}  // namespace orbit

using namespace orbit;

namespace orbit {

static void free_graphs(orbit_program_t* p) {
  cudaGraphExec_t* gs[] = {&p->g_first, &p->g_mid, &p->g_last, &p->g_single};
  for (auto g : gs)
    if (*g) { cudaGraphExecDestroy(*g); *g = nullptr; }
}

static bool sync_equal(const orbit_sync_t& a, const orbit_sync_t& b) {
  return a.beta == b.beta && a.gamma == b.gamma && a.momentum == b.momentum && a.charge == b.charge &&
         a.classical_radius == b.classical_radius && a.macrosize == b.macrosize && a.mass == b.mass;
}

KickArgs kick_args(orbit_sc2p5d_t* c, const orbit_sync_t& s, double length, const orbit_boundary* bnd) {
  KickArgs ka;
  ka.st = c->d_st;
  ka.phi = c->d_phi;
  ka.lam = c->d_lam;
  ka.phi_f = c->d_phi_f;
  ka.lam_f = c->d_lam_f;
  ka.phi_fix = c->d_phi_fix;
  ka.lam_fix = c->d_lam_fix;
  ka.host_factor = sc_host_factor(s, length);
  ka.nx = c->nx; ka.ny = c->ny; ka.nz = c->nz; ka.form = c->form;
  ka.lamd = c->rb ? c->d_lamd : nullptr;
  ka.rb_lsf = c->rb ? sc_rb_long_factor(s, length) : 0.0;
  ka.bnd = bnd_shape_of(bnd);
  return ka;
}

// One fused pass: optional kick of calculator kc, maps [a,b), optional
// extrema for calculator ec.
// ec_here: the kick of ec is enqueued next in this same stream (and graph),
// so a graph branch for its Green rebuild can be set up by this pass.
static int enqueue_pass(orbit_bunch_t* bu, cudaStream_t s, const DevOp* ops, Seg seg, const MapCtx& m,
                        orbit_sc2p5d_t* kc, double klen, const orbit_boundary* kb, orbit_sc2p5d_t* ec,
                        const orbit_boundary* eb, bool ec_here, double* knl_buf, int km, int* nl) {
  KickArgs ka;
  std::memset(&ka, 0, sizeof(ka));
  int kf = 0;
  size_t smem = 0;
  bool ksm = false;
  if (kc) {
    ka = kick_args(kc, bu->sync, klen, kb);
    kf = kc->form == ORBIT_FORM_PLAIN ? 1 : 2;
    smem = (kf == 1 ? 8 : 4) * ((size_t)kc->nx * kc->ny + kc->nz);
    ksm = kc->smem_kick && smem <= (size_t)kPassSmem;  // else the kick reads phi_fix, converted by the solve
  }
  if (!kc && !ec && seg.a == seg.b) return ORBIT_OK;  // nothing to do
  ScState* ext = ec ? ec->d_st : nullptr;
  bool e = ext != nullptr;
  SetupArgs sa;
  std::memset(&sa, 0, sizeof(sa));
  if (ec) {
    sa = sc_setup_args(ec, sc_dep_scales(ec, bu), eb);
    if (ec_here) sa.cond = sc_green_cond(ec, s, true);
  }
  int rc;
  if (kf == 0) rc = e ? launch_pass<0, true, false>(bu, s, 0, ops, seg.a, seg.b, m, ka, ext, sa, knl_buf, km)
                      : launch_pass<0, false, false>(bu, s, 0, ops, seg.a, seg.b, m, ka, ext, sa, knl_buf, km);
  else if (kf == 1) {
    if (ksm) rc = e ? launch_pass<1, true, true>(bu, s, smem, ops, seg.a, seg.b, m, ka, ext, sa, knl_buf, km)
                    : launch_pass<1, false, true>(bu, s, smem, ops, seg.a, seg.b, m, ka, ext, sa, knl_buf, km);
    else rc = e ? launch_pass<1, true, false>(bu, s, 0, ops, seg.a, seg.b, m, ka, ext, sa, knl_buf, km)
                : launch_pass<1, false, false>(bu, s, 0, ops, seg.a, seg.b, m, ka, ext, sa, knl_buf, km);
  } else {
    if (ksm) rc = e ? launch_pass<2, true, true>(bu, s, smem, ops, seg.a, seg.b, m, ka, ext, sa, knl_buf, km)
                    : launch_pass<2, false, true>(bu, s, smem, ops, seg.a, seg.b, m, ka, ext, sa, knl_buf, km);
    else rc = e ? launch_pass<2, true, false>(bu, s, 0, ops, seg.a, seg.b, m, ka, ext, sa, knl_buf, km)
                : launch_pass<2, false, false>(bu, s, 0, ops, seg.a, seg.b, m, ka, ext, sa, knl_buf, km);
  }
  if (rc == ORBIT_OK) ++*nl;
  return rc;
}

// Builds the device op array: all non-SC ops of the turn in order, then the
// wrap segment (last segment followed by the first).
int compile(orbit_program_t* p, orbit_bunch_t* bu, Plan& plan) {
  std::vector<DevOp> dev;
  p->time_adv.assign(p->ops.size(), 0.0);
  int start = 0;
  std::vector<std::pair<int, int>> seg_ops;  // [first op, last op) in p->ops for each segment
  for (size_t k = 0; k < p->ops.size(); ++k) {
    if (p->ops[k].code == ORBIT_OP_SC) {
      seg_ops.push_back({start, (int)k});
      plan.sc_idx.push_back((int)k);
      start = (int)k + 1;
    }
  }
  seg_ops.push_back({start, (int)p->ops.size()});
  // Maps that add to x, y and z a term linear in their length and change
  // neither xp, yp nor dE (drift; quad2 = bend2) compose by adding lengths:
  // drift(L1) drift(L2) = drift(L1+L2) and quad2(L1) quad2(L2) =
  // quad2(L1+L2), equal in exact arithmetic (each reads only xp, yp and
  // dp_p, which the other leaves alone), one rounding per coordinate instead
  // of two.  The reference's quad schedule issues quad2(L) twice in a row
  // when the element has no multipoles (teapot.py:945-960).
  auto lengthwise = [](int code) {
    return code == ORBIT_OP_DRIFT ? 1 : (code == ORBIT_OP_QUAD2 || code == ORBIT_OP_BEND2) ? 2 : 0;
  };
  auto emit = [&](int a, int b) -> Seg {
    Seg s;
    s.a = (int)dev.size();
    s.dE = false;
    for (int k = a; k < b; ++k) {
      DevOp d;
      double adv = 0.0;
      if (!compile_op(p->ops[k], bu->sync, d, &adv)) return Seg{-1, -1, false};
      p->time_adv[k] = adv;
      if (d.code == ORBIT_OP_WEDGEROT || (d.code == ORBIT_OP_KICK && d.c[2] != 0.)) s.dE = true;
      if (d.code == 0) continue;
      if (lengthwise(d.code) && (int)dev.size() > s.a && lengthwise(dev.back().code) == lengthwise(d.code)) {
        dev.back().c[0] += d.c[0];
        continue;
      }
      dev.push_back(d);
    }
    s.b = (int)dev.size();
    return s;
  };
  for (auto& so : seg_ops) {
    Seg s = emit(so.first, so.second);
    if (s.a < 0) return set_error(ORBIT_ERR_ARG, "orbit_program: bad op parameters");
    plan.segs.push_back(s);
  }
  Seg w;
  w.a = (int)dev.size();
  {
    Seg s1 = emit(seg_ops.back().first, seg_ops.back().second);
    Seg s2 = emit(seg_ops.front().first, seg_ops.front().second);
    if (s1.a < 0 || s2.a < 0) return set_error(ORBIT_ERR_ARG, "orbit_program: bad op parameters");
  }
  w.b = (int)dev.size();
  w.dE = plan.segs.back().dE || plan.segs.front().dE;
  plan.wrap = w;
  if (p->knl_n < (size_t)bu->n) {
    if (p->d_knl) { cudaFree(p->d_knl); p->d_knl = nullptr; }
    p->knl_n = 0;
    if (bu->n > 0) {
      ORBIT_CUDA(cudaMalloc(&p->d_knl, sizeof(double) * (size_t)bu->n));
      p->knl_n = (size_t)bu->n;
    }
  }
  if (p->d_ops) { cudaFree(p->d_ops); p->d_ops = nullptr; }
  p->n_devops = (int)dev.size();
  if (!dev.empty()) {
    ORBIT_CUDA(cudaMalloc(&p->d_ops, sizeof(DevOp) * dev.size()));
    ORBIT_CUDA(cudaMemcpy(p->d_ops, dev.data(), sizeof(DevOp) * dev.size(), cudaMemcpyHostToDevice));
  }
  return ORBIT_OK;
}

// Enqueues one turn.  prologue: run P_0 first.  wrap: end with the pass
// that also applies M_0 of the next turn and its extrema scan.
static int enqueue_turn(orbit_program_t* p, orbit_bunch_t* bu, cudaStream_t s, const Plan& plan, bool prologue,
                        bool wrap, int* nl) {
  const DevOp* ops = p->d_ops;
  MapCtx m = make_ctx(bu->sync);
  int nsc = (int)plan.sc_idx.size();
  bool sc_active = bu->n >= 2;  // SpaceChargeCalc2p5D.cc:79-80
  auto calc_of = [&](int i) -> orbit_sc2p5d_t* { return p->calcs[p->ops[plan.sc_idx[i]].i0]; };
  auto len_of = [&](int i) -> double { return p->ops[plan.sc_idx[i]].d[0]; };
  auto pipe_of = [&](int i) -> double { return p->ops[plan.sc_idx[i]].d[1]; };
  int rc;
  // the first pass of the run stores 1/(1+dp_p); later passes load it and
  // store it again only when their ops change dE
  bool first = true;
  // (a 2.5Drb kick at the start of a pass also changes dE)
  auto km_of = [&](const Seg& sg, bool sc, orbit_sc2p5d_t* kc = nullptr) -> int {
    if (!sc && sg.a == sg.b) return 0;  // enqueue_pass launches nothing
    bool dE = sg.dE || (kc && kc->rb);
    int km = first ? (int)KNL_STORE : (KNL_LOAD | (dE ? KNL_STORE : 0));
    first = false;
    return km;
  };
  double* knl = p->d_knl;
  auto bnd_of = [&](int i) -> const orbit_boundary* {
    int k = p->ops[plan.sc_idx[i]].i1;
    return (k >= 1 && k <= (int)p->bnds.size()) ? p->bnds[k - 1] : nullptr;
  };
  if (nsc == 0 || !sc_active) {
    // no kicks: one pass over all maps of the turn
    for (size_t i = 0; i < plan.segs.size(); ++i) {
      rc = enqueue_pass(bu, s, ops, plan.segs[i], m, nullptr, 0.0, nullptr, nullptr, nullptr, false, knl,
                        km_of(plan.segs[i], false), nl);
      if (rc) return rc;
    }
    return ORBIT_OK;
  }
  if (prologue) {
    rc = enqueue_pass(bu, s, ops, plan.segs[0], m, nullptr, 0.0, nullptr, calc_of(0), bnd_of(0), true, knl,
                      km_of(plan.segs[0], true), nl);
    if (rc) return rc;
  }
  for (int i = 0; i < nsc; ++i) {
    rc = sc_enqueue_kick(calc_of(i), bu, len_of(i), s, false, false, nl, pipe_of(i), bnd_of(i));
    if (rc) return rc;
    bool last = (i == nsc - 1);
    if (!last) {
      rc = enqueue_pass(bu, s, ops, plan.segs[i + 1], m, calc_of(i), len_of(i), bnd_of(i), calc_of(i + 1),
                        bnd_of(i + 1), true, knl, km_of(plan.segs[i + 1], true, calc_of(i)), nl);
    } else if (wrap) {
      rc = enqueue_pass(bu, s, ops, plan.wrap, m, calc_of(i), len_of(i), bnd_of(i), calc_of(0), bnd_of(0), false,
                        knl, km_of(plan.wrap, true, calc_of(i)), nl);
    } else {
      rc = enqueue_pass(bu, s, ops, plan.segs[nsc], m, calc_of(i), len_of(i), bnd_of(i), nullptr, nullptr, false,
                        knl, km_of(plan.segs[nsc], true, calc_of(i)), nl);
    }
    if (rc) return rc;
  }
  return ORBIT_OK;
}

static int capture(orbit_program_t* p, orbit_bunch_t* bu, const Plan& plan, bool prologue, bool wrap,
                   cudaGraphExec_t* out, int* nl) {
  cudaStream_t s = bu->stream;
  for (auto c : p->calcs) sc_clear_pending(c);
  ORBIT_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_turn(p, bu, s, plan, prologue, wrap, nl);
  for (auto c : p->calcs) sc_clear_pending(c);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_error(e, "cudaGraphInstantiate");
  return ORBIT_OK;
}

static int prepare(orbit_program_t* p, orbit_bunch_t* bu) {
  auto dnv = [](const orbit_sc2p5d_t* c) { return c && c->dn ? dn_version(c->dn) : 0ull; };
  bool same = p->key_bunch == bu && p->key_n == bu->n && p->key_coords == bu->d_coords &&
              p->key_msize == bu->has_msize && sync_equal(p->key_sync, bu->sync) && p->g_mid &&
              p->key_gen.size() == p->calcs.size() && p->key_dnv.size() == p->calcs.size();
  for (size_t i = 0; same && i < p->calcs.size(); ++i)
    same = p->key_gen[i] == (p->calcs[i] ? p->calcs[i]->cfg_gen : 0ull) && p->key_dnv[i] == dnv(p->calcs[i]);
  if (same) return ORBIT_OK;
  free_graphs(p);
  for (auto c : p->calcs)
    if (c && c->dn) {
      int prc = dn_prepare_capture(c->dn);
      if (prc) return prc;
    }
  Plan plan;
  int rc = compile(p, bu, plan);
  if (rc) return rc;
  int nl = 0;
  rc = capture(p, bu, plan, true, true, &p->g_first, &nl);
  if (!rc) { nl = 0; rc = capture(p, bu, plan, false, true, &p->g_mid, &nl); }
  if (!rc) { p->launches_per_turn = nl; nl = 0; rc = capture(p, bu, plan, false, false, &p->g_last, &nl); }
  if (!rc) { nl = 0; rc = capture(p, bu, plan, true, false, &p->g_single, &nl); }
  if (rc) { free_graphs(p); return rc; }
  p->key_bunch = bu;
  p->key_n = bu->n;
  p->key_coords = bu->d_coords;
  p->key_sync = bu->sync;
  p->key_msize = bu->has_msize;
  p->key_gen.resize(p->calcs.size());
  p->key_dnv.resize(p->calcs.size());
  for (size_t i = 0; i < p->calcs.size(); ++i) {
    p->key_gen[i] = p->calcs[i] ? p->calcs[i]->cfg_gen : 0ull;
    p->key_dnv[i] = dnv(p->calcs[i]);
  }
  return ORBIT_OK;
}

}  // namespace orbit

extern "C" {

int orbit_program_create(orbit_program_t** out, const orbit_op_t* ops, int nops, orbit_sc2p5d_t* const* calcs,
                         int ncalcs) {
  if (!out || nops < 0 || (nops > 0 && !ops) || ncalcs < 0 || (ncalcs > 0 && !calcs))
    return set_error(ORBIT_ERR_ARG, "orbit_program_create: bad argument");
  int arc = init_pass_attrs();
  if (arc) return arc;
  num_sms();
  orbit_program_t* p = new orbit_program_t();
  p->ops.assign(ops, ops + nops);
  p->calcs.assign(calcs, calcs + ncalcs);
  for (auto& o : p->ops) {
    if (o.code == ORBIT_OP_SC && (o.i0 < 0 || o.i0 >= ncalcs || !p->calcs[o.i0])) {
      delete p;
      return set_error(ORBIT_ERR_ARG, "orbit_program_create: SC op refers to a missing calculator");
    }
  }
  cudaError_t e = cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    delete p;
    return cuda_error(e, "orbit_program_create");
  }
  *out = p;
  return ORBIT_OK;
}

int orbit_program_set_boundaries(orbit_program_t* p, orbit_boundary_t* const* bnds, int n) {
  if (!p || n < 0 || (n > 0 && !bnds)) return set_error(ORBIT_ERR_ARG, "orbit_program_set_boundaries: bad argument");
  for (int i = 0; i < n; ++i) {
    int init = 0;
    if (!bnds[i] || orbit_boundary_info(bnds[i], nullptr, nullptr, nullptr, nullptr, &init) || !init)
      return set_error(ORBIT_ERR_ARG, "Boundary2D: the boundary was not initialized, call initialize()");
    int rc = bnd_ensure_device(bnds[i]);
    if (rc) return rc;
  }
  if (p->used) ORBIT_CUDA(cudaEventSynchronize(p->done));
  p->bnds.assign(bnds, bnds + n);
  free_graphs(p);
  p->key_bunch = nullptr;
  return ORBIT_OK;
}

int orbit_program_destroy(orbit_program_t* p) {
  if (!p) return ORBIT_OK;
  if (p->used) cudaEventSynchronize(p->done);  // graphs in flight read d_ops
  if (p->done) cudaEventDestroy(p->done);
  free_graphs(p);
  if (p->d_ops) cudaFree(p->d_ops);
  if (p->d_knl) cudaFree(p->d_knl);
  delete p;
  return ORBIT_OK;
}

int orbit_program_run(orbit_program_t* p, orbit_bunch_t* b, int turns) {
  int rc = orbit_program_enqueue(p, b, turns);
  if (rc) return rc;
  return check_status(b);
}

int orbit_program_enqueue(orbit_program_t* p, orbit_bunch_t* b, int turns) {
  ORBIT_NVTX("lattice program turns");
  if (!p || !b || turns < 0) return set_error(ORBIT_ERR_ARG, "orbit_program_enqueue: bad argument");
  if (turns == 0) return ORBIT_OK;
  // work already queued on a calculator by another bunch comes first
  for (auto c : p->calcs)
    ORBIT_CUDA(sc_order_before(c, b->stream));
  int rc = prepare(p, b);
  if (rc) return rc;
  if (turns == 1) {
    ORBIT_CUDA(cudaGraphLaunch(p->g_single, b->stream));
  } else {
    ORBIT_CUDA(cudaGraphLaunch(p->g_first, b->stream));
    for (int t = 1; t < turns - 1; ++t) ORBIT_CUDA(cudaGraphLaunch(p->g_mid, b->stream));
    ORBIT_CUDA(cudaGraphLaunch(p->g_last, b->stream));
  }
  for (auto c : p->calcs) ORBIT_CUDA(sc_mark_used(c, b->stream));
  p->used = true;
  ORBIT_CUDA(cudaEventRecord(p->done, b->stream));
  // SyncPart time, advanced in op order as each map would (teapotbase.cc:165)
  for (int t = 0; t < turns; ++t)
    for (double a : p->time_adv)
      if (a != 0.0) b->sync.time = b->sync.time + a;
  return ORBIT_OK;
}

int orbit_program_profile(orbit_program_t* p, orbit_bunch_t* b, int max_kinds, char* names, double* total_ms,
                          int* launches, int* nkinds) {
  if (!p || !b || max_kinds <= 0 || !names || !total_ms || !launches || !nkinds)
    return set_error(ORBIT_ERR_ARG, "orbit_program_profile: bad argument");
  for (auto c : p->calcs)
    ORBIT_CUDA(sc_order_before(c, b->stream));
  // an eager (uncaptured) turn; the captured graphs are rebuilt on the next run
  ORBIT_CUDA(cudaStreamSynchronize(b->stream));
  free_graphs(p);
  p->key_bunch = nullptr;
  Plan plan;
  int rc = compile(p, b, plan);
  if (rc) return rc;
  Profiler* prof = prof_install();
  int nl = 0;
  rc = enqueue_turn(p, b, b->stream, plan, true, false, &nl);
  int rc2 = prof_collect(prof, max_kinds, names, total_ms, launches, nkinds);
  for (auto c : p->calcs) ORBIT_CUDA(sc_mark_used(c, b->stream));
  for (double a : p->time_adv)
    if (a != 0.0) b->sync.time = b->sync.time + a;
  if (rc) return rc;
  if (rc2) return rc2;
  return check_status(b);
}

int orbit_program_launches(const orbit_program_t* p, int* launches) {
  if (!p || !launches) return set_error(ORBIT_ERR_ARG, "orbit_program_launches: bad argument");
  *launches = p->launches_per_turn;
  return ORBIT_OK;
}

}  // extern "C"
