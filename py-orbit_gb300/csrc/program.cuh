// Lattice programs (program.cu): the recorded op list, its compiled device
// form and the captured turn graphs; shared with the batched executor
// (batch.cu).
#pragma once

#include <vector>

#include "sc2p5d.cuh"
#include "teapot.cuh"

struct orbit_program {
  std::vector<orbit_op_t> ops;
  std::vector<orbit_sc2p5d_t*> calcs;
  std::vector<orbit_boundary_t*> bnds;   // SC ops with i1 = 1 + index
  // compiled for one bunch configuration
  orbit_bunch_t* key_bunch = nullptr;
  int key_n = -1;
  double* key_coords = nullptr;
  orbit_sync_t key_sync{};
  int key_msize = -1;
  std::vector<unsigned long long> key_gen;  // the calculators' cfg_gen
  std::vector<unsigned long long> key_dnv;  // their networks' parameter versions
  orbit::DevOp* d_ops = nullptr;
  int n_devops = 0;
  double* d_knl = nullptr;            // per-particle 1/(1+dp_p) between passes
  size_t knl_n = 0;
  cudaGraphExec_t g_first = nullptr;  // prologue + turn ending with the wrap pass
  cudaGraphExec_t g_mid = nullptr;    // turn ending with the wrap pass
  cudaGraphExec_t g_last = nullptr;   // turn ending without the wrap
  cudaGraphExec_t g_single = nullptr; // prologue + turn without wrap (one-turn runs)
  std::vector<double> time_adv;       // per-op SyncPart time increments
  int launches_per_turn = 0;
  cudaEvent_t done = nullptr;         // recorded after the last enqueued run
  bool used = false;
};

namespace orbit {

struct Seg {
  int a, b;
  bool dE;  // an op of the segment changes dE (kick with dE, wedgerotate)
};

struct Plan {
  std::vector<Seg> segs;      // m+1 map segments in the device op array
  std::vector<int> sc_idx;    // op index of each SC op
  Seg wrap;                   // M_m ++ M_0 in the device op array
};

// Per-particle 1/(1+dp_p) kept between the passes of one program run
// (it changes only with dE): km & KNL_STORE writes it at the end of the
// pass, km & KNL_LOAD reads it instead of dividing.
enum { KNL_LOAD = 1, KNL_STORE = 2 };

// Builds the device op array of the program for the bunch's reference
// particle: all non-SC ops of the turn in order, then the wrap segment.
int compile(orbit_program_t* p, orbit_bunch_t* bu, Plan& plan);
// Kick arguments of calculator c for a kick of `length`.
KickArgs kick_args(orbit_sc2p5d_t* c, const orbit_sync_t& s, double length, const orbit_boundary* bnd);
int check_status(orbit_bunch_t* b);

}  // namespace orbit
