// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// C-ABI harness over the UNMODIFIED reference C++ (PyORBIT src/orbit,
// src/spacecharge, src/teapot), compiled in place from the reference tree by
// oracle/build_ref.sh into oracle/_ref/.  It replaces the Python-2 wrappers
// (src/spacecharge/wrap_spacechargecalc2p5d.cc, src/teapot/wrap_teapotbase.cc,
// src/orbit/wrap_bunch.cc, src/orbit/wrap_syncpart.cc) so that ctypes can
// drive the reference's own hot path from Python 3.  It is used only to pin
// the CPU restatement (oracle/orbit_oracle.c) and to generate golden vectors;
// it never ships in the product library and cannot run on the GPU host
// (the reference tree is not there).
#include "Bunch.hh"
#include "SyncPart.hh"
#include "SpaceChargeCalc2p5D.hh"
#include "SpaceChargeCalc2p5Drb.hh"
#include "ShapedBoundary2D.hh"
#include "BunchTwissAnalysis.hh"
#include "BunchTuneAnalysis.hh"
#include "ParticleAttributes.hh"
#include <map>
#include <string>
#include "Grid1D.hh"
#include "Grid2D.hh"
#include "teapotbase.hh"

#include <cstdlib>

// The reference's Bunch() asks the Python MPI-comm wrapper for a
// communicator (src/orbit/Bunch.cc:59,107).  Without MPI and without the
// Python-2 wrapper module, a heap object holding MPI_COMM_WORLD stands in.
namespace wrap_orbit_mpi_comm {
pyORBIT_MPI_Comm* newMPI_Comm() {
  pyORBIT_MPI_Comm* c = (pyORBIT_MPI_Comm*)calloc(1, sizeof(pyORBIT_MPI_Comm));
  c->comm = MPI_COMM_WORLD;
  return c;
}
void freeMPI_Comm(pyORBIT_MPI_Comm* c) { free(c); }
}  // namespace wrap_orbit_mpi_comm

extern "C" {

void* ref_bunch_new() {
  teapot_base::init_factorial();
  return new Bunch();
}
void ref_bunch_free(void* b) { delete (Bunch*)b; }

// Same steps as SyncPart_kinEnergy(value) (src/orbit/wrap_syncpart.cc:70-93).
double ref_bunch_set_kin_energy(void* b, double ek) {
  SyncPart* s = ((Bunch*)b)->getSyncPart();
  double p = s->energyToMomentum(ek);
  s->setMomentum(p);
  return s->momentumToEnergy(p);
}
void ref_bunch_set_macrosize(void* b, double m) { ((Bunch*)b)->setMacroSize(m); }
void ref_bunch_set_mass(void* b, double m) { ((Bunch*)b)->setMass(m); }
void ref_bunch_set_charge(void* b, double c) { ((Bunch*)b)->setCharge(c); }
int ref_bunch_size(void* b) { return ((Bunch*)b)->getSize(); }

// kin[0..6] = beta, gamma, momentum, kinetic energy, mass, classical radius, time
void ref_bunch_kinematics(void* b, double* kin) {
  Bunch* bb = (Bunch*)b;
  SyncPart* s = bb->getSyncPart();
  kin[0] = s->getBeta();
  kin[1] = s->getGamma();
  kin[2] = s->getMomentum();
  kin[3] = s->getEnergy();
  kin[4] = bb->getMass();
  kin[5] = bb->getClassicalRadius();
  kin[6] = s->getTime();
}

// soa: x[n], xp[n], y[n], yp[n], z[n], dE[n]
void ref_bunch_add(void* b, int n, const double* soa) {
  Bunch* bb = (Bunch*)b;
  for (int i = 0; i < n; ++i)
    bb->addParticle(soa[i], soa[n + i], soa[2 * n + i], soa[3 * n + i], soa[4 * n + i], soa[5 * n + i]);
}
void ref_bunch_get(void* b, double* soa) {
  Bunch* bb = (Bunch*)b;
  int n = bb->getSize();
  double** a = bb->coordArr();
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 6; ++c) soa[c * n + i] = a[i][c];
}
void ref_bunch_set(void* b, const double* soa) {
  Bunch* bb = (Bunch*)b;
  int n = bb->getSize();
  double** a = bb->coordArr();
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 6; ++c) a[i][c] = soa[c * n + i];
}

// Bunch text I/O as the Python wrapper drives it (src/orbit/wrap_bunch.cc:
// dumpBunch -> Bunch::print(fileName), readBunch -> initBunchAttributes,
// readParticleAttributes, readBunchCoords), and the attribute calls a
// golden bunch file needs.
void ref_bunch_dump(void* b, const char* fn) { ((Bunch*)b)->print(fn); }
void ref_bunch_read(void* b, const char* fn) {
  Bunch* bb = (Bunch*)b;
  bb->initBunchAttributes(fn);
  bb->readParticleAttributes(fn);
  bb->readBunchCoords(fn);
}
void ref_bunch_add_attr(void* b, const char* name, int size) {
  std::map<std::string, double> d;
  if (size > 0) d["size"] = size;
  ((Bunch*)b)->addParticleAttributes(std::string(name), d);
}
int ref_bunch_attr_size(void* b, const char* name) {
  ParticleAttributes* a = ((Bunch*)b)->getParticleAttributes(std::string(name));
  return a ? a->getAttSize() : -1;
}
void ref_bunch_attr_set(void* b, const char* name, int i, int j, double v) {
  ((Bunch*)b)->getParticleAttributes(std::string(name))->attValue(i, j) = v;
}
double ref_bunch_attr_get(void* b, const char* name, int i, int j) {
  return ((Bunch*)b)->getParticleAttributes(std::string(name))->attValue(i, j);
}
void ref_bunch_set_int_attr(void* b, const char* name, int v) { ((Bunch*)b)->setBunchAttribute(std::string(name), v); }
void ref_bunch_set_double_attr(void* b, const char* name, double v) {
  ((Bunch*)b)->setBunchAttribute(std::string(name), v);
}
int ref_bunch_get_int_attr(void* b, const char* name) { return ((Bunch*)b)->getBunchAttributeInt(std::string(name)); }
double ref_bunch_get_double_attr(void* b, const char* name) {
  return ((Bunch*)b)->getBunchAttributeDouble(std::string(name));
}
void ref_bunch_set_time(void* b, double t) { ((Bunch*)b)->getSyncPart()->setTime(t); }

// Same constructor choice as SpaceChargeCalc2p5D_init
// (src/spacecharge/wrap_spacechargecalc2p5d.cc:38-52).
void* ref_sc_new(int nx, int ny, int nz, double xy_ratio) {
  if (xy_ratio > 0.) return new SpaceChargeCalc2p5D(nx, ny, nz, xy_ratio);
  return new SpaceChargeCalc2p5D(nx, ny, nz);
}
void ref_sc_free(void* sc) { delete (SpaceChargeCalc2p5D*)sc; }
void ref_sc_track(void* sc, void* b, double length) {
  ((SpaceChargeCalc2p5D*)sc)->trackBunch((Bunch*)b, length, NULL);
}
// rho/phi: nx*ny row-major [ix][iy]; zg: nz; lim: xmin,xmax,ymin,ymax,zmin,zmax,dx,dy,dz
void ref_sc_grids(void* sc, double* rho, double* phi, double* zg, double* lim) {
  SpaceChargeCalc2p5D* c = (SpaceChargeCalc2p5D*)sc;
  Grid2D* r = c->getRhoGrid();
  Grid2D* p = c->getPhiGrid();
  Grid1D* z = c->getLongGrid();
  int nx = r->getSizeX(), ny = r->getSizeY();
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      rho[i * ny + j] = r->getValueOnGrid(i, j);
      phi[i * ny + j] = p->getValueOnGrid(i, j);
    }
  for (int k = 0; k < z->getSizeZ(); ++k) zg[k] = z->getValueOnGrid(k);
  lim[0] = r->getMinX(); lim[1] = r->getMaxX();
  lim[2] = r->getMinY(); lim[3] = r->getMaxY();
  lim[4] = z->getMinZ(); lim[5] = z->getMaxZ();
  lim[6] = r->getStepX(); lim[7] = r->getStepY(); lim[8] = z->getStepZ();
}
// Per-particle gradient of the current phi grid and lambda(z), as the kick
// loop evaluates them (src/spacecharge/SpaceChargeCalc2p5D.cc:104-119).
void ref_sc_fields(void* sc, int n, const double* x, const double* y, const double* z,
                   double* ex, double* ey, double* lam) {
  SpaceChargeCalc2p5D* c = (SpaceChargeCalc2p5D*)sc;
  Grid2D* p = c->getPhiGrid();
  Grid1D* zg = c->getLongGrid();
  for (int i = 0; i < n; ++i) {
    p->calcGradient(x[i], y[i], ex[i], ey[i]);
    lam[i] = zg->getValue(z[i]);
  }
}

// ---- bunch diagnostics (src/orbit/BunchDiagnostics) ----
// BunchTwissAnalysis::analyzeBunch, then out = {count, total macrosize,
// <c_i> [6], getCorrelation(i, j) for i >= j [21]} and the
// getters g = {emittance, normalized, alpha, beta, gamma} x {x, y, z},
// dispersion and its derivative x, y, effective {emittance, alpha, beta,
// gamma} x, y.
void ref_twiss(void* b, double* out, double* g) {
  BunchTwissAnalysis t;
  t.analyzeBunch((Bunch*)b);
  out[0] = t.getGlobalCount();
  out[1] = t.getGlobalMacrosize();
  for (int i = 0; i < 6; ++i) out[2 + i] = t.getAverage(i);
  int k = 8;
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j <= i; ++j) out[k++] = t.getCorrelation(i, j);
  k = 0;
  for (int ic = 0; ic < 3; ++ic) {
    g[k++] = t.getEmittance(ic);
    g[k++] = t.getEmittanceNormalized(ic);
    g[k++] = t.getAlpha(ic);
    g[k++] = t.getBeta(ic);
    g[k++] = t.getGamma(ic);
  }
  for (int ic = 0; ic < 2; ++ic) {
    g[k++] = t.getDispersion(ic);
    g[k++] = t.getDispersionDerivative(ic);
    g[k++] = t.getEffectiveEmittance(ic);
    g[k++] = t.getEffectiveAlpha(ic);
    g[k++] = t.getEffectiveBeta(ic);
    g[k++] = t.getEffectiveGamma(ic);
  }
}
// BunchTwissAnalysis::computeBunchMoments then getBunchMoment(i, j) for
// i, j = 0..order into out[i * (order + 1) + j] (order >= 2: for order 1 the
// reference writes outside its table).
void ref_bunch_moments(void* b, int order, int dispersion, int emitnorm, double* out) {
  BunchTwissAnalysis t;
  t.computeBunchMoments((Bunch*)b, order, dispersion, emitnorm);
  for (int i = 0; i <= order; ++i)
    for (int j = 0; j <= order; ++j) out[i * (order + 1) + j] = t.getBunchMoment(i, j);
}
void* ref_tune_new() { return new BunchTuneAnalysis(); }
void ref_tune_free(void* t) { delete (BunchTuneAnalysis*)t; }
void ref_tune_assign(void* t, const double* tw) {
  ((BunchTuneAnalysis*)t)->assignTwiss(tw[0], tw[1], tw[2], tw[3], tw[4], tw[5]);
}
// analyzeBunch, then the six attribute rows (SoA of n)
void ref_tune_analyze(void* t, void* b, double* ph) {
  Bunch* bunch = (Bunch*)b;
  ((BunchTuneAnalysis*)t)->analyzeBunch(bunch);
  int n = bunch->getSize();
  ParticleAttributes* a = bunch->getParticleAttributes("ParticlePhaseAttributes");
  for (int k = 0; k < 6; ++k)
    for (int i = 0; i < n; ++i) ph[(size_t)k * n + i] = a->attValue(i, k);
}

// ---- boundaries (src/spacecharge/BaseBoundary2D.cc, ShapedBoundary2D.cc) ----
// As Boundary2D_init (src/spacecharge/wrap_boundary2d.cc:37-68): shape 0
// selects BaseBoundary2D(nPoints, nModes), 1/2/3 ShapedBoundary2D with
// "Circle"/"Ellipse"/"Rectangle".
void* ref_bnd_new(int np, int nm, int shape, double xdim, double ydim) {
  if (shape == 0) return new BaseBoundary2D(np, nm);
  const char* names[] = {"", "Circle", "Ellipse", "Rectangle"};
  return new ShapedBoundary2D(np, nm, std::string(names[shape]), xdim, ydim);
}
void ref_bnd_free(void* b) { delete (BaseBoundary2D*)b; }
void ref_bnd_set_point(void* b, int i, double x, double y) { ((BaseBoundary2D*)b)->setBoundaryPoint(i, x, y); }
void ref_bnd_initialize(void* b) { ((BaseBoundary2D*)b)->initializeBPs(); }
int ref_bnd_is_inside(void* b, double x, double y) { return ((BaseBoundary2D*)b)->isInside(x, y); }
// head = {np, nm, xmin, xmax, ymin, ymax}; bx, by [np]
void ref_bnd_get(void* b, double* head, double* bx, double* by) {
  BaseBoundary2D* q = (BaseBoundary2D*)b;
  int np = q->getNumberOfPoints();
  head[0] = np; head[1] = q->getNumberOfModes();
  head[2] = q->getMinX(); head[3] = q->getMaxX(); head[4] = q->getMinY(); head[5] = q->getMaxY();
  for (int i = 0; i < np; ++i) { bx[i] = q->getBoundaryPointX(i); by[i] = q->getBoundaryPointY(i); }
}
void ref_sc_track_bnd(void* sc, void* b, double length, void* bnd) {
  ((SpaceChargeCalc2p5D*)sc)->trackBunch((Bunch*)b, length, (BaseBoundary2D*)bnd);
}

// ---- SpaceChargeCalc2p5Drb (src/spacecharge/SpaceChargeCalc2p5Drb.cc) ----
// Same constructor choice as SpaceChargeCalc2p5Drb_init
// (src/spacecharge/wrap_spacechargecalc2p5d_rb.cc:37-50).
void* ref_scrb_new(int nx, int ny, int nz, double xy_ratio) {
  if (xy_ratio > 0.) return new SpaceChargeCalc2p5Drb(nx, ny, nz, xy_ratio);
  return new SpaceChargeCalc2p5Drb(nx, ny, nz);
}
void ref_scrb_free(void* sc) { delete (SpaceChargeCalc2p5Drb*)sc; }
void ref_scrb_set_long_avg(void* sc, int n) { ((SpaceChargeCalc2p5Drb*)sc)->setLongAveragingPointsN(n); }
void ref_scrb_track(void* sc, void* b, double length, double pipe_radius) {
  ((SpaceChargeCalc2p5Drb*)sc)->trackBunch((Bunch*)b, length, pipe_radius);
}
// rho, phi [nx*ny], zg, zderiv [nz], lim as ref_sc_grids
void ref_scrb_grids(void* sc, double* rho, double* phi, double* zg, double* zd, double* lim) {
  SpaceChargeCalc2p5Drb* c = (SpaceChargeCalc2p5Drb*)sc;
  Grid2D* r = c->getRhoGrid();
  Grid2D* p = c->getPhiGrid();
  Grid1D* z = c->getLongGrid();
  Grid1D* d = c->getLongDerivativeGrid();
  int nx = r->getSizeX(), ny = r->getSizeY();
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      rho[i * ny + j] = r->getValueOnGrid(i, j);
      phi[i * ny + j] = p->getValueOnGrid(i, j);
    }
  for (int k = 0; k < z->getSizeZ(); ++k) {
    zg[k] = z->getValueOnGrid(k);
    zd[k] = d->getValueOnGrid(k);
  }
  lim[0] = r->getMinX(); lim[1] = r->getMaxX();
  lim[2] = r->getMinY(); lim[3] = r->getMaxY();
  lim[4] = z->getMinZ(); lim[5] = z->getMaxZ();
  lim[6] = r->getStepX(); lim[7] = r->getStepY(); lim[8] = z->getStepZ();
}

// ---- teapot_base maps (src/teapot/teapotbase.cc) ----
void ref_tpb_rotatexy(void* b, double a) { teapot_base::rotatexy((Bunch*)b, a); }
void ref_tpb_drift(void* b, double L) { teapot_base::drift((Bunch*)b, L); }
void ref_tpb_wrapbunch(void* b, double L) { teapot_base::wrapbunch((Bunch*)b, L); }
void ref_tpb_kick(void* b, double kx, double ky, double kE) { teapot_base::kick((Bunch*)b, kx, ky, kE, 1); }
void ref_tpb_multp(void* b, int pole, double kl, int skew) { teapot_base::multp((Bunch*)b, pole, kl, skew, 1); }
void ref_tpb_multpfringeIN(void* b, int pole, double kl, int skew) { teapot_base::multpfringeIN((Bunch*)b, pole, kl, skew, 1); }
void ref_tpb_multpfringeOUT(void* b, int pole, double kl, int skew) { teapot_base::multpfringeOUT((Bunch*)b, pole, kl, skew, 1); }
void ref_tpb_quad1(void* b, double L, double kq) { teapot_base::quad1((Bunch*)b, L, kq, 1); }
void ref_tpb_quad2(void* b, double L) { teapot_base::quad2((Bunch*)b, L); }
void ref_tpb_quadfringeIN(void* b, double kq) { teapot_base::quadfringeIN((Bunch*)b, kq, 1); }
void ref_tpb_quadfringeOUT(void* b, double kq) { teapot_base::quadfringeOUT((Bunch*)b, kq, 1); }
void ref_tpb_wedgerotate(void* b, double e, int fr) { teapot_base::wedgerotate((Bunch*)b, e, fr); }
void ref_tpb_wedgedrift(void* b, double e, int io) { teapot_base::wedgedrift((Bunch*)b, e, io); }
void ref_tpb_wedgebend(void* b, double e, int io, double rho, int ns) { teapot_base::wedgebend((Bunch*)b, e, io, rho, ns); }
void ref_tpb_bend1(void* b, double L, double th) { teapot_base::bend1((Bunch*)b, L, th); }
void ref_tpb_bend2(void* b, double L) { teapot_base::bend2((Bunch*)b, L); }
void ref_tpb_bend3(void* b, double th) { teapot_base::bend3((Bunch*)b, th); }
void ref_tpb_bend4(void* b, double th) { teapot_base::bend4((Bunch*)b, th); }
void ref_tpb_bendfringeIN(void* b, double rho) { teapot_base::bendfringeIN((Bunch*)b, rho); }
void ref_tpb_bendfringeOUT(void* b, double rho) { teapot_base::bendfringeOUT((Bunch*)b, rho); }

}  // extern "C"
