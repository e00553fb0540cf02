// Batched lattice tracking: many independent bunches (the points of an
// intensity or quadrupole-strength scan), each with its own lattice program
// and 2.5D calculator, advance together, turn by turn.  Members are grouped
// into classes of equal grid size; every stage of a kick interval (Green
// rebuild, deposit, Poisson solve, fused kick + maps + extrema pass) is one
// launch for all members of a class, and each class runs on its own stream
// inside one captured CUDA graph per turn.
//
// Per class an autotuner picks the launch shapes: the deposit's and the
// pass's threads and particles per block, timed live on the first turn (any
// shape gives the same result: the deposit sums integers, the pass is per
// particle), and the FFT stage schedule (radix-2 stages with N/2 threads or
// radix-4 stages with N/4 threads; the two differ in rounding only), timed on
// the class's own work buffers before the first turn.
//
// The members' programs must share one node structure (the same op codes and
// SC nodes in the same places; strengths, lengths of the kicks and reference
// particles may differ), use one plain-form 2.5D calculator each (no
// boundary, no 2.5Drb) and track at least two particles.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "batch.cuh"
#include "program.cuh"

namespace orbit {

// Candidate launch shapes of the particle kernels.
static const int kDepCand[][2] = {{768, 4096}, {768, 8192}, {768, 16384}, {768, 32768}, {512, 8192}};
static const int kNDep = 5;
#ifndef ORBIT_PASS_THREADS
#define ORBIT_PASS_THREADS 512
#endif
static const int kPassCand[][2] = {{ORBIT_PASS_THREADS, 2048}, {ORBIT_PASS_THREADS, 4096}, {ORBIT_PASS_THREADS, 8192},
                                   {ORBIT_PASS_THREADS, 16384}};
static const int kNPass = 4;

struct BatchClass {
  int nx = 0, ny = 0, nz = 0;
  std::vector<int> mem;            // member indices
  orbit_sc2p5d_t* proto = nullptr;
  ClassTuning tune{};
  bool ksmem = false;              // the kick keeps a copy of the potential in shared memory
  size_t kick_smem = 0;
  SolveJob* d_solve = nullptr;
  DepJob* d_dep = nullptr;
  PassJob* d_pass = nullptr;       // (nsc + 1) tables of mem.size() jobs: [0] no kick, [1 + i] kick i
  std::vector<BlockMap> dep_maps;  // one per deposit candidate
  std::vector<BlockMap> pass_maps; // one per pass candidate
  int dep_sel = 0, pass_sel = 0;
  std::string dep_tag, pass_tag;   // profile names of the class's deposit and kick passes
  cudaStream_t st = nullptr;
  cudaEvent_t joined = nullptr;
};

// Timing of the candidate shapes over the first turn.
struct Tuner {
  struct Rec {
    int cls, stage, cand;  // stage 0 deposit, 1 pass
    cudaEvent_t a, b;
  };
  std::vector<Rec> recs;
  ~Tuner() {
    for (auto& r : recs) {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
  }
};

}  // namespace orbit

using namespace orbit;

struct orbit_batch {
  std::vector<orbit_program_t*> progs;
  std::vector<orbit_bunch_t*> bunches;
  std::vector<orbit_sc2p5d_t*> calcs;
  Plan plan;                        // common to all members
  std::vector<BatchClass> classes;
  int nsc = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  bool used = false;
  bool tuned = false;               // shapes chosen (a tuning turn ran or they were set)
  bool fft_probed = false;
  // compiled for these bunch configurations
  std::vector<int> key_n, key_ms;
  std::vector<double*> key_coords;
  std::vector<orbit_sync_t> key_sync;
  std::vector<DevOp*> key_ops;      // the members' compiled ops (a program recompiled alone frees them)
  bool compiled = false;
  cudaGraphExec_t g_first = nullptr, g_mid = nullptr, g_last = nullptr, g_single = nullptr;
  int launches_per_turn = 0;
};

namespace orbit {

static void free_map(BlockMap& m) {
  if (m.blk_job) cudaFree(m.blk_job);
  if (m.mblk) cudaFree(m.mblk);
  m = BlockMap{};
}

static void free_tables(BatchClass& c) {
  if (c.d_solve) cudaFree(c.d_solve);
  if (c.d_dep) cudaFree(c.d_dep);
  if (c.d_pass) cudaFree(c.d_pass);
  c.d_solve = nullptr;
  c.d_dep = nullptr;
  c.d_pass = nullptr;
  for (auto& m : c.dep_maps) free_map(m);
  for (auto& m : c.pass_maps) free_map(m);
  c.dep_maps.clear();
  c.pass_maps.clear();
}

static void free_graphs(orbit_batch_t* bt) {
  cudaGraphExec_t* gs[] = {&bt->g_first, &bt->g_mid, &bt->g_last, &bt->g_single};
  for (auto g : gs)
    if (*g) { cudaGraphExecDestroy(*g); *g = nullptr; }
}

static bool sync_same(const orbit_sync_t& a, const orbit_sync_t& b) {
  return a.beta == b.beta && a.gamma == b.gamma && a.momentum == b.momentum && a.charge == b.charge &&
         a.classical_radius == b.classical_radius && a.macrosize == b.macrosize && a.mass == b.mass;
}

// Blocks of each member for `chunk` particles per `per` blocks.
static int build_map(const orbit_batch_t* bt, const BatchClass& c, int chunk, int per, BlockMap& out) {
  std::vector<unsigned short> bj;
  std::vector<int2> mb(c.mem.size());
  for (size_t j = 0; j < c.mem.size(); ++j) {
    int n = bt->bunches[c.mem[j]]->n;
    int nb = (n + chunk - 1) / chunk;
    if (nb < 1) nb = 1;
    nb *= per;
    mb[j].x = (int)bj.size();
    mb[j].y = nb;
    bj.insert(bj.end(), (size_t)nb, (unsigned short)j);
  }
  if (bj.size() > (size_t)0x7fffffff) return set_error(ORBIT_ERR_UNSUPPORTED, "orbit_batch: too many blocks");
  ORBIT_CUDA(cudaMalloc(&out.blk_job, sizeof(unsigned short) * bj.size()));
  ORBIT_CUDA(cudaMalloc(&out.mblk, sizeof(int2) * mb.size()));
  ORBIT_CUDA(cudaMemcpy(out.blk_job, bj.data(), sizeof(unsigned short) * bj.size(), cudaMemcpyHostToDevice));
  ORBIT_CUDA(cudaMemcpy(out.mblk, mb.data(), sizeof(int2) * mb.size(), cudaMemcpyHostToDevice));
  out.nblk = (int)bj.size();
  return ORBIT_OK;
}

template <typename J>
static int upload(J** dst, const std::vector<J>& v) {
  ORBIT_CUDA(cudaMalloc(dst, sizeof(J) * v.size()));
  ORBIT_CUDA(cudaMemcpy(*dst, v.data(), sizeof(J) * v.size(), cudaMemcpyHostToDevice));
  return ORBIT_OK;
}

// Job tables of one class for the members' current bunches and reference
// particles.
static int build_tables(orbit_batch_t* bt, BatchClass& c) {
  free_tables(c);
  const size_t nm = c.mem.size();
  std::vector<SolveJob> sj(nm);
  std::vector<DepJob> dj(nm);
  std::vector<PassJob> pj((size_t)(bt->nsc + 1) * nm);
  for (size_t j = 0; j < nm; ++j) {
    const int m = c.mem[j];
    orbit_sc2p5d_t* k = bt->calcs[m];
    orbit_bunch_t* b = bt->bunches[m];
    orbit_program_t* p = bt->progs[m];
    SolveJob& S = sj[j];
    S.st = k->d_st;
    S.rho_q = k->d_rho_q;
    S.z_q = k->d_z_q;
    S.rho = k->d_rho;
    S.lam = k->d_lam;
    S.phi = k->d_phi;
    S.gbuf = k->d_gbuf;
    S.hat = (double2*)k->d_hat;
    S.green = (double2*)k->d_green;
    S.tw_x = (const double2*)k->d_tw_x;
    S.tw_y = (const double2*)k->d_tw_y;
    S.phi_fix = k->d_phi_fix;
    S.lam_fix = k->d_lam_fix;
    const DepScales ds = sc_dep_scales(k, b);
    DepJob& D = dj[j];
    D.x = b->coord(0);
    D.y = b->coord(2);
    D.z = b->coord(4);
    D.msize = b->has_msize ? b->d_msize : nullptr;
    D.n = b->n;
    D.K = ds.K;
    D.st = k->d_st;
    D.g_rho = k->d_rho_q;
    D.g_z = k->d_z_q;
    D.ms_uniform = ds.ms_uniform;
    D.qscale = ds.S;
    SetupArgs sa = sc_setup_args(k, ds, nullptr);
    sa.cond = 0;
    for (int t = 0; t <= bt->nsc; ++t) {
      PassJob& P = pj[(size_t)t * nm + j];
      std::memset(&P, 0, sizeof(P));
      for (int q = 0; q < 6; ++q) P.c[q] = b->coord(q);
      P.n = b->n;
      P.ops = p->d_ops;
      P.m = make_ctx(b->sync);
      if (t > 0) P.ka = kick_args(k, b->sync, p->ops[bt->plan.sc_idx[t - 1]].d[0], nullptr);
      P.ext = k->d_st;
      P.status = b->d_status;
      P.sa = sa;
      P.knl = p->d_knl;
    }
  }
  int rc = upload(&c.d_solve, sj);
  if (!rc) rc = upload(&c.d_dep, dj);
  if (!rc) rc = upload(&c.d_pass, pj);
  if (rc) return rc;
  c.dep_maps.resize(kNDep);
  c.pass_maps.resize(kNPass);
  const int bands = batch_deposit_bands(c.proto);
  for (int q = 0; q < kNDep && !rc; ++q) rc = build_map(bt, c, kDepCand[q][1], bands, c.dep_maps[q]);
  for (int q = 0; q < kNPass && !rc; ++q) rc = build_map(bt, c, kPassCand[q][1], 1, c.pass_maps[q]);
  return rc;
}

// Compiles every member's program for its bunch and checks that they share
// one structure; rebuilds the job tables.
static int compile_all(orbit_batch_t* bt) {
  const size_t nmem = bt->progs.size();
  std::vector<Plan> plans(nmem);
  for (size_t m = 0; m < nmem; ++m) {
    orbit_program_t* p = bt->progs[m];
    if (p->used) ORBIT_CUDA(cudaEventSynchronize(p->done));  // its own graphs in flight read p->d_ops
    int rc = compile(p, bt->bunches[m], plans[m]);
    if (rc) return rc;
    p->key_bunch = nullptr;  // the program recompiles and recaptures before it runs alone again
  }
  auto same_seg = [](const Seg& a, const Seg& b) { return a.a == b.a && a.b == b.b && a.dE == b.dE; };
  for (size_t m = 1; m < nmem; ++m) {
    bool ok = plans[m].segs.size() == plans[0].segs.size() && plans[m].sc_idx == plans[0].sc_idx &&
              same_seg(plans[m].wrap, plans[0].wrap);
    for (size_t i = 0; ok && i < plans[m].segs.size(); ++i) ok = same_seg(plans[m].segs[i], plans[0].segs[i]);
    if (ok) {
      // the same op codes in the same places
      std::vector<DevOp> a(bt->progs[0]->n_devops), b(bt->progs[m]->n_devops);
      ok = a.size() == b.size();
      if (ok && !a.empty()) {
        ORBIT_CUDA(cudaMemcpy(a.data(), bt->progs[0]->d_ops, sizeof(DevOp) * a.size(), cudaMemcpyDeviceToHost));
        ORBIT_CUDA(cudaMemcpy(b.data(), bt->progs[m]->d_ops, sizeof(DevOp) * b.size(), cudaMemcpyDeviceToHost));
        for (size_t q = 0; ok && q < a.size(); ++q) ok = a[q].code == b[q].code;
      }
    }
    if (!ok) return set_error(ORBIT_ERR_ARG, "orbit_batch: the members' lattices differ in structure");
  }
  bt->plan = plans[0];
  bt->nsc = (int)bt->plan.sc_idx.size();
  for (auto& c : bt->classes) {
    int rc = build_tables(bt, c);
    if (rc) return rc;
  }
  bt->key_n.resize(nmem);
  bt->key_ms.resize(nmem);
  bt->key_coords.resize(nmem);
  bt->key_sync.resize(nmem);
  bt->key_ops.resize(nmem);
  for (size_t m = 0; m < nmem; ++m) {
    orbit_bunch_t* b = bt->bunches[m];
    bt->key_ops[m] = bt->progs[m]->d_ops;
    bt->key_n[m] = b->n;
    bt->key_ms[m] = b->has_msize;
    bt->key_coords[m] = b->d_coords;
    bt->key_sync[m] = b->sync;
  }
  bt->compiled = true;
  return ORBIT_OK;
}

static bool key_same(const orbit_batch_t* bt) {
  if (!bt->compiled) return false;
  for (size_t m = 0; m < bt->bunches.size(); ++m) {
    const orbit_bunch_t* b = bt->bunches[m];
    if (b->n != bt->key_n[m] || b->has_msize != bt->key_ms[m] || b->d_coords != bt->key_coords[m] ||
        !sync_same(b->sync, bt->key_sync[m]) || bt->progs[m]->d_ops != bt->key_ops[m])
      return false;
  }
  return true;
}

static int rec_begin(Tuner* tu, int cls, int stage, int cand, cudaStream_t s, Tuner::Rec* r) {
  if (!tu) return ORBIT_OK;
  r->cls = cls;
  r->stage = stage;
  r->cand = cand;
  ORBIT_CUDA(cudaEventCreate(&r->a));
  ORBIT_CUDA(cudaEventCreate(&r->b));
  ORBIT_CUDA(cudaEventRecord(r->a, s));
  return ORBIT_OK;
}

static int rec_end(Tuner* tu, cudaStream_t s, Tuner::Rec& r) {
  if (!tu) return ORBIT_OK;
  ORBIT_CUDA(cudaEventRecord(r.b, s));
  tu->recs.push_back(r);
  return ORBIT_OK;
}

// One turn of one class on stream s.  With a tuner the particle kernels of
// kick interval i use candidate shapes i mod (number of candidates).
static int enqueue_class_turn(orbit_batch_t* bt, int ci, cudaStream_t s, bool prologue, bool wrap, Tuner* tu,
                              int* nl) {
  BatchClass& c = bt->classes[ci];
  const int nm = (int)c.mem.size();
  const int nsc = bt->nsc;
  const Plan& plan = bt->plan;
  bool first = true;
  auto km_of = [&](const Seg& sg) -> int {
    int km = first ? (int)KNL_STORE : (KNL_LOAD | (sg.dE ? KNL_STORE : 0));
    first = false;
    return km;
  };
  // (only kick passes are timed: the prologue pass has no kick)
  auto pass = [&](int table, const Seg& sg, bool kick, bool ext, int cand) -> int {
    Tuner* t = kick ? tu : nullptr;
    Tuner::Rec r{};
    int rc = rec_begin(t, ci, 1, cand, s, &r);
    if (rc) return rc;
    rc = batch_enqueue_pass(c.d_pass + (size_t)table * nm, c.pass_maps[cand], kPassCand[cand][0], kick ? 1 : 0, ext,
                            kick && c.ksmem, c.kick_smem, sg.a, sg.b, km_of(sg), s, c.pass_tag.c_str());
    if (rc) return rc;
    ++*nl;
    return rec_end(t, s, r);
  };
  int rc;
  if (prologue) {
    rc = pass(0, plan.segs[0], false, true, c.pass_sel);
    if (rc) return rc;
  }
  for (int i = 0; i < nsc; ++i) {
    rc = batch_enqueue_green(c.d_solve, nm, c.proto, c.tune.fft_wide, s);
    if (rc) return rc;
    *nl += 3;
    int dc = tu ? i % kNDep : c.dep_sel;
    Tuner::Rec r{};
    rc = rec_begin(tu, ci, 0, dc, s, &r);
    if (!rc) rc = batch_enqueue_deposit(c.d_dep, c.dep_maps[dc], c.proto, kDepCand[dc][0], s, c.dep_tag.c_str());
    if (!rc) rc = rec_end(tu, s, r);
    if (rc) return rc;
    ++*nl;
    rc = batch_enqueue_solve(c.d_solve, nm, c.proto, c.tune.fft_wide, !c.ksmem, s);
    if (rc) return rc;
    *nl += c.ksmem ? 3 : 4;
    int pc = tu ? i % kNPass : c.pass_sel;
    bool last = i == nsc - 1;
    if (!last) rc = pass(1 + i, plan.segs[i + 1], true, true, pc);
    else if (wrap) rc = pass(1 + i, plan.wrap, true, true, pc);
    else rc = pass(1 + i, plan.segs[nsc], true, false, pc);
    if (rc) return rc;
  }
  return ORBIT_OK;
}

// One turn of every class: forked onto the class streams, joined on the
// batch stream; `serial` (the tuning and the profiled turns) runs the
// classes one after another on the batch stream.
static int enqueue_turn(orbit_batch_t* bt, bool prologue, bool wrap, Tuner* tu, int* nl, bool serial = false) {
  if (tu || serial) {
    for (size_t ci = 0; ci < bt->classes.size(); ++ci) {
      int rc = enqueue_class_turn(bt, (int)ci, bt->stream, prologue, wrap, tu, nl);
      if (rc) return rc;
    }
    return ORBIT_OK;
  }
  ORBIT_CUDA(cudaEventRecord(bt->fork, bt->stream));
  for (size_t ci = 0; ci < bt->classes.size(); ++ci) {
    BatchClass& c = bt->classes[ci];
    ORBIT_CUDA(cudaStreamWaitEvent(c.st, bt->fork, 0));
    int rc = enqueue_class_turn(bt, (int)ci, c.st, prologue, wrap, nullptr, nl);
    if (rc) return rc;
    ORBIT_CUDA(cudaEventRecord(c.joined, c.st));
    ORBIT_CUDA(cudaStreamWaitEvent(bt->stream, c.joined, 0));
  }
  return ORBIT_OK;
}

static int capture(orbit_batch_t* bt, bool prologue, bool wrap, cudaGraphExec_t* out, int* nl) {
  ORBIT_CUDA(cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_turn(bt, prologue, wrap, nullptr, nl);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(bt->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_error(e, "orbit_batch: cudaStreamEndCapture");
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_error(e, "orbit_batch: cudaGraphInstantiate");
  return ORBIT_OK;
}

static int capture_all(orbit_batch_t* bt) {
  free_graphs(bt);
  int nl = 0;
  int rc = capture(bt, true, true, &bt->g_first, &nl);
  if (!rc) { nl = 0; rc = capture(bt, false, true, &bt->g_mid, &nl); }
  if (!rc) { bt->launches_per_turn = nl; nl = 0; rc = capture(bt, false, false, &bt->g_last, &nl); }
  if (!rc) { nl = 0; rc = capture(bt, true, false, &bt->g_single, &nl); }
  if (rc) free_graphs(bt);
  return rc;
}

// FFT schedule of each class: the column transforms with the Green multiply
// and the backward rows, timed with both schedules on the class's own work
// spectra and potentials (overwritten by the next solve; max |phi| is reset
// by the next grid set-up) before the first turn.
static int probe_fft(orbit_batch_t* bt) {
  cudaEvent_t a, b;
  ORBIT_CUDA(cudaEventCreate(&a));
  ORBIT_CUDA(cudaEventCreate(&b));
  int rc = ORBIT_OK;
  for (auto& c : bt->classes) {
    if (!c.proto->plan_x.pow2 && !c.proto->plan_y.pow2) {
      c.tune.fft_wide = 1;
      continue;
    }
    float best[2] = {1e30f, 1e30f};
    for (int rep = 0; rep < 3 && !rc; ++rep) {
      for (int w = 0; w < 2 && !rc; ++w) {
        int wide = (rep & 1) ? 1 - w : w;
        if (cudaEventRecord(a, bt->stream) != cudaSuccess) { rc = cuda_error(cudaGetLastError(), "probe"); break; }
        rc = batch_enqueue_fft_probe(c.d_solve, (int)c.mem.size(), c.proto, wide, bt->stream);
        if (rc) break;
        cudaEventRecord(b, bt->stream);
        cudaError_t e = cudaEventSynchronize(b);
        if (e != cudaSuccess) { rc = cuda_error(e, "orbit_batch: FFT probe"); break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0) best[wide] = std::min(best[wide], ms);
      }
    }
    c.tune.fft_wide = best[1] <= best[0] ? 1 : 0;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return rc;
}

// Median time of each candidate shape over the tuning turn; the fastest
// is kept.
static int finish_tuning(orbit_batch_t* bt, Tuner& tu) {
  ORBIT_CUDA(cudaStreamSynchronize(bt->stream));
  std::map<std::tuple<int, int, int>, std::vector<float>> t;
  for (auto& r : tu.recs) {
    float ms = 0.f;
    ORBIT_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
    t[std::make_tuple(r.cls, r.stage, r.cand)].push_back(ms);
  }
  for (size_t ci = 0; ci < bt->classes.size(); ++ci) {
    BatchClass& c = bt->classes[ci];
    for (int stage = 0; stage < 2; ++stage) {
      int nc = stage == 0 ? kNDep : kNPass;
      int best = 0;
      float bv = 1e30f;
      for (int q = 0; q < nc; ++q) {
        auto it = t.find(std::make_tuple((int)ci, stage, q));
        if (it == t.end() || it->second.empty()) continue;
        std::vector<float> v = it->second;
        std::sort(v.begin(), v.end());
        float med = v[v.size() / 2];
        if (med < bv) { bv = med; best = q; }
      }
      if (stage == 0) c.dep_sel = best;
      else c.pass_sel = best;
    }
    c.tune.dep_threads = kDepCand[c.dep_sel][0];
    c.tune.dep_chunk = kDepCand[c.dep_sel][1];
    c.tune.pass_threads = kPassCand[c.pass_sel][0];
    c.tune.pass_chunk = kPassCand[c.pass_sel][1];
  }
  bt->tuned = true;
  return ORBIT_OK;
}

static int order_in(orbit_batch_t* bt) {
  // the members' earlier work (uploads, single-bunch tracking) comes first
  for (auto b : bt->bunches) {
    ORBIT_CUDA(cudaEventRecord(bt->done, b->stream));
    ORBIT_CUDA(cudaStreamWaitEvent(bt->stream, bt->done, 0));
  }
  for (auto c : bt->calcs) ORBIT_CUDA(sc_order_before(c, bt->stream));
  return ORBIT_OK;
}

static int order_out(orbit_batch_t* bt, int turns) {
  for (auto c : bt->calcs) ORBIT_CUDA(sc_mark_used(c, bt->stream));
  ORBIT_CUDA(cudaEventRecord(bt->done, bt->stream));
  for (auto b : bt->bunches) ORBIT_CUDA(cudaStreamWaitEvent(b->stream, bt->done, 0));
  bt->used = true;
  // SyncPart time of each member, advanced in op order (teapotbase.cc:165)
  for (size_t m = 0; m < bt->bunches.size(); ++m)
    for (int t = 0; t < turns; ++t)
      for (double a : bt->progs[m]->time_adv)
        if (a != 0.0) bt->bunches[m]->sync.time = bt->bunches[m]->sync.time + a;
  return ORBIT_OK;
}

}  // namespace orbit

extern "C" {

int orbit_batch_create(orbit_batch_t** out, orbit_program_t* const* progs, orbit_bunch_t* const* bunches, int n) {
  if (!out || n <= 0 || !progs || !bunches) return set_error(ORBIT_ERR_ARG, "orbit_batch_create: bad argument");
  if (n > 65535) return set_error(ORBIT_ERR_UNSUPPORTED, "orbit_batch_create: at most 65535 members");
  std::vector<orbit_sc2p5d_t*> calcs(n);
  for (int m = 0; m < n; ++m) {
    orbit_program_t* p = progs[m];
    if (!p || !bunches[m]) return set_error(ORBIT_ERR_ARG, "orbit_batch_create: null member");
    for (int q = 0; q < m; ++q)
      if (bunches[q] == bunches[m] || progs[q] == progs[m])
        return set_error(ORBIT_ERR_ARG, "orbit_batch_create: a bunch or program appears twice");
    orbit_sc2p5d_t* c = nullptr;
    for (auto& o : p->ops) {
      if (o.code != ORBIT_OP_SC) continue;
      orbit_sc2p5d_t* k = p->calcs[o.i0];
      if (c && k != c) return set_error(ORBIT_ERR_ARG, "orbit_batch_create: a member uses more than one calculator");
      c = k;
      if (o.i1 != 0) return set_error(ORBIT_ERR_UNSUPPORTED, "orbit_batch_create: boundaries are not batched");
    }
    if (!c) return set_error(ORBIT_ERR_ARG, "orbit_batch_create: a member's lattice has no SC node");
    if (c->form != ORBIT_FORM_PLAIN || c->rb)
      return set_error(ORBIT_ERR_UNSUPPORTED, "orbit_batch_create: only plain-form 2.5D calculators are batched");
    for (int q = 0; q < m; ++q)
      if (calcs[q] == c) return set_error(ORBIT_ERR_ARG, "orbit_batch_create: members share a calculator");
    calcs[m] = c;
  }
  orbit_batch_t* bt = new orbit_batch_t();
  bt->progs.assign(progs, progs + n);
  bt->bunches.assign(bunches, bunches + n);
  bt->calcs = calcs;
  // classes by grid size, in order of first appearance
  for (int m = 0; m < n; ++m) {
    orbit_sc2p5d_t* c = calcs[m];
    BatchClass* cls = nullptr;
    for (auto& k : bt->classes)
      if (k.nx == c->nx && k.ny == c->ny && k.nz == c->nz) cls = &k;
    if (!cls) {
      bt->classes.emplace_back();
      cls = &bt->classes.back();
      cls->nx = c->nx;
      cls->ny = c->ny;
      cls->nz = c->nz;
      cls->proto = c;
      cls->kick_smem = 8 * ((size_t)c->nx * c->ny + c->nz);
      cls->ksmem = c->smem_kick && cls->kick_smem <= batch_pass_smem_limit();
      cls->tune = ClassTuning{kDepCand[1][0], kDepCand[1][1], kPassCand[1][0], kPassCand[1][1], 1};
      std::string g = std::to_string(c->nx) + "x" + std::to_string(c->ny) + "x" + std::to_string(c->nz);
      cls->dep_tag = "batch_deposit_" + g;
      cls->pass_tag = "batch_pass_" + g;
      cls->dep_sel = 1;
      cls->pass_sel = 1;
    }
    cls->mem.push_back(m);
  }
  int rc = ORBIT_OK;
  auto fail = [&](int code) {
    orbit_batch_destroy(bt);
    return code;
  };
  for (auto& c : bt->classes) {
    rc = batch_init_attrs(c.proto);
    if (rc) return fail(rc);
    if (cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c.joined, cudaEventDisableTiming) != cudaSuccess)
      return fail(cuda_error(cudaGetLastError(), "orbit_batch_create"));
  }
  if (cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&bt->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&bt->done, cudaEventDisableTiming) != cudaSuccess)
    return fail(cuda_error(cudaGetLastError(), "orbit_batch_create"));
  *out = bt;
  return ORBIT_OK;
}

int orbit_batch_destroy(orbit_batch_t* bt) {
  if (!bt) return ORBIT_OK;
  if (bt->stream) cudaStreamSynchronize(bt->stream);
  free_graphs(bt);
  for (auto& c : bt->classes) {
    free_tables(c);
    if (c.st) cudaStreamDestroy(c.st);
    if (c.joined) cudaEventDestroy(c.joined);
  }
  if (bt->fork) cudaEventDestroy(bt->fork);
  if (bt->done) cudaEventDestroy(bt->done);
  if (bt->stream) cudaStreamDestroy(bt->stream);
  delete bt;
  return ORBIT_OK;
}

int orbit_batch_enqueue(orbit_batch_t* bt, int turns) {
  ORBIT_NVTX("batch turns");
  if (!bt || turns < 0) return set_error(ORBIT_ERR_ARG, "orbit_batch_enqueue: bad argument");
  if (turns == 0) return ORBIT_OK;
  for (auto b : bt->bunches)
    if (b->n < 2) return set_error(ORBIT_ERR_ARG, "orbit_batch: every member needs at least two particles");
  int rc = order_in(bt);
  if (rc) return rc;
  if (!key_same(bt)) {
    ORBIT_CUDA(cudaStreamSynchronize(bt->stream));  // graphs in flight read the old tables
    free_graphs(bt);
    rc = compile_all(bt);
    if (rc) return rc;
  }
  int done_turns = 0;
  if (!bt->tuned) {
    if (!bt->fft_probed) {
      rc = probe_fft(bt);
      if (rc) return rc;
      bt->fft_probed = true;
    }
    // the first turn runs uncaptured and times the candidate shapes
    Tuner tu;
    int nl = 0;
    rc = enqueue_turn(bt, true, turns > 1, &tu, &nl);
    if (rc) return rc;
    rc = finish_tuning(bt, tu);
    if (rc) return rc;
    done_turns = 1;
  }
  if (!bt->g_mid) {
    rc = capture_all(bt);
    if (rc) return rc;
  }
  int left = turns - done_turns;
  if (left > 0) {
    if (done_turns == 1) {
      // the tuning turn ended with the wrap pass
      for (int t = 0; t < left - 1; ++t) ORBIT_CUDA(cudaGraphLaunch(bt->g_mid, bt->stream));
      ORBIT_CUDA(cudaGraphLaunch(bt->g_last, bt->stream));
    } else if (left == 1) {
      ORBIT_CUDA(cudaGraphLaunch(bt->g_single, bt->stream));
    } else {
      ORBIT_CUDA(cudaGraphLaunch(bt->g_first, bt->stream));
      for (int t = 1; t < left - 1; ++t) ORBIT_CUDA(cudaGraphLaunch(bt->g_mid, bt->stream));
      ORBIT_CUDA(cudaGraphLaunch(bt->g_last, bt->stream));
    }
  }
  return order_out(bt, turns);
}

int orbit_batch_sync(orbit_batch_t* bt) {
  if (!bt) return set_error(ORBIT_ERR_ARG, "orbit_batch_sync: bad argument");
  ORBIT_CUDA(cudaStreamSynchronize(bt->stream));
  int first = ORBIT_OK;
  for (auto b : bt->bunches) {
    int rc = check_status(b);
    if (rc && !first) first = rc;
  }
  return first;
}

int orbit_batch_run(orbit_batch_t* bt, int turns) {
  int rc = orbit_batch_enqueue(bt, turns);
  if (rc) return rc;
  return orbit_batch_sync(bt);
}

int orbit_batch_stream(orbit_batch_t* bt, void** stream) {
  if (!bt || !stream) return set_error(ORBIT_ERR_ARG, "orbit_batch_stream: bad argument");
  *stream = (void*)bt->stream;
  return ORBIT_OK;
}

int orbit_batch_profile(orbit_batch_t* bt, int max_kinds, char* names, double* total_ms, int* launches,
                        int* nkinds) {
  if (!bt || max_kinds <= 0 || !names || !total_ms || !launches || !nkinds)
    return set_error(ORBIT_ERR_ARG, "orbit_batch_profile: bad argument");
  if (!bt->tuned) return set_error(ORBIT_ERR_ARG, "orbit_batch_profile: run the batch once first (autotuning)");
  for (auto b : bt->bunches)
    if (b->n < 2) return set_error(ORBIT_ERR_ARG, "orbit_batch: every member needs at least two particles");
  int rc = order_in(bt);
  if (rc) return rc;
  if (!key_same(bt)) {
    ORBIT_CUDA(cudaStreamSynchronize(bt->stream));
    free_graphs(bt);
    rc = compile_all(bt);
    if (rc) return rc;
  }
  ORBIT_CUDA(cudaStreamSynchronize(bt->stream));
  Profiler* prof = prof_install();
  int nl = 0;
  rc = enqueue_turn(bt, true, false, nullptr, &nl, true);
  int rc2 = prof_collect(prof, max_kinds, names, total_ms, launches, nkinds);
  int rc3 = order_out(bt, 1);
  if (rc) return rc;
  if (rc2) return rc2;
  if (rc3) return rc3;
  return orbit_batch_sync(bt);
}

int orbit_batch_info(const orbit_batch_t* bt, int* n_classes, int* launches_per_turn) {
  if (!bt) return set_error(ORBIT_ERR_ARG, "orbit_batch_info: bad argument");
  if (n_classes) *n_classes = (int)bt->classes.size();
  if (launches_per_turn) *launches_per_turn = bt->launches_per_turn;
  return ORBIT_OK;
}

int orbit_batch_class(const orbit_batch_t* bt, int cls, int* grid, int* members, int* tuning) {
  if (!bt || cls < 0 || cls >= (int)bt->classes.size()) return set_error(ORBIT_ERR_ARG, "orbit_batch_class: bad class");
  const BatchClass& c = bt->classes[cls];
  if (grid) { grid[0] = c.nx; grid[1] = c.ny; grid[2] = c.nz; }
  if (members) *members = (int)c.mem.size();
  if (tuning) {
    tuning[0] = c.tune.dep_threads;
    tuning[1] = c.tune.dep_chunk;
    tuning[2] = c.tune.pass_threads;
    tuning[3] = c.tune.pass_chunk;
    tuning[4] = c.tune.fft_wide;
    tuning[5] = bt->tuned ? 1 : 0;
  }
  return ORBIT_OK;
}

int orbit_batch_set_tuning(orbit_batch_t* bt, int cls, const int* tuning) {
  if (!bt || !tuning || cls < 0 || cls >= (int)bt->classes.size())
    return set_error(ORBIT_ERR_ARG, "orbit_batch_set_tuning: bad argument");
  BatchClass& c = bt->classes[cls];
  int ds = -1, ps = -1;
  for (int q = 0; q < kNDep; ++q)
    if (kDepCand[q][0] == tuning[0] && kDepCand[q][1] == tuning[1]) ds = q;
  for (int q = 0; q < kNPass; ++q)
    if (kPassCand[q][0] == tuning[2] && kPassCand[q][1] == tuning[3]) ps = q;
  if (ds < 0 || ps < 0 || (tuning[4] != 0 && tuning[4] != 1))
    return set_error(ORBIT_ERR_ARG, "orbit_batch_set_tuning: not one of the candidate shapes");
  if (bt->used) ORBIT_CUDA(cudaStreamSynchronize(bt->stream));
  c.dep_sel = ds;
  c.pass_sel = ps;
  c.tune = ClassTuning{tuning[0], tuning[1], tuning[2], tuning[3], tuning[4]};
  // the shapes of every class are fixed once one is set by hand
  bt->tuned = true;
  bt->fft_probed = true;
  free_graphs(bt);
  return ORBIT_OK;
}

}  // extern "C"
