// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// C API over the reference's own classes, built from the reference sources (see Makefile).
// It reproduces the driver call sequences of sphericalVertex.cpp:87-125 (Brownian) and
// minimization.cpp:245-264 (FIRE) so tests can run the unmodified reference CPU path and
// compare the oracle restatement and the GPU path against it.
#include <memory>
#include <vector>
#include <cstring>
#include "std_include.h"
#include "sphericalVertexModel.h"
#include "brownianDynamics.h"
#include "energyMinimizerFIRE.h"
#include "simulation.h"
#include "noiseSource.h"
#include "hyperrectangularCellList.h"
#include "neighborList.h"
#include "sphericalSelfPropelledParticle.h"
#include "sphericalVectorialVicsek.h"
#include "dynamicalFeatures.h"
#include "simpleUtilities.h"

struct ref_handle {
    noiseSource initNoise{true};
    std::shared_ptr<sphericalVertexModel> model;
    std::shared_ptr<brownianDynamics> bd;
    std::shared_ptr<energyMinimizerFIRE> fire;
    std::shared_ptr<Simulation> sim;
    std::shared_ptr<vectorialVicsek> active;   // the self-propelled or Vicsek updater
};

extern "C" {

// sphericalVertex.cpp:88-90 with noise.setReproducibleSeed(seed) (minimization.cpp:245)
ref_handle* ref_create(int nCells, int seed, double a0, double p0, double kr, double t1) {
    ref_handle* h = new ref_handle();
    if (seed >= 0) h->initNoise.setReproducibleSeed(seed);
    h->model = std::make_shared<sphericalVertexModel>(nCells, h->initNoise, a0, p0, false, true);
    h->model->setScalarModelParameter(kr);
    h->model->setT1Threshold(t1);
    return h;
}
void ref_destroy(ref_handle* h) { delete h; }

// sphericalVertex.cpp:92-102 (BD with its own noise, seeded when bdSeed >= 0)
void ref_bd_setup(ref_handle* h, int bdSeed, double T, double dt, double mu) {
    h->bd = std::make_shared<brownianDynamics>(true);
    h->sim = std::make_shared<Simulation>();
    h->sim->setConfiguration(h->model);
    h->sim->addUpdater(h->bd, h->model);
    h->sim->setIntegrationTimestep(dt);
    h->sim->setCPUOperation(true);
    h->sim->setReproducible(true);
    if (bdSeed >= 0) h->bd->noise.setReproducibleSeed(bdSeed);
    h->bd->setT(T);
    h->bd->mu = mu;
}

// An active updater on the model, as mainwindow.cpp:184-214 wires the self-propelled one:
// kind 0 sphericalSelfPropelledParticle, 1 sphericalVectorialVicsek; the updater's own noise
// seeded with `seed`.
void ref_active_setup(ref_handle* h, int kind, int seed, double dt, double mu, double v0, double eta, double tau) {
    if (kind == 0) h->active = std::make_shared<sphericalSelfPropelledParticle>();
    else h->active = std::make_shared<sphericalVectorialVicsek>();
    h->sim = std::make_shared<Simulation>();
    h->sim->setConfiguration(h->model);
    h->sim->addUpdater(h->active, h->model);
    h->sim->setIntegrationTimestep(dt);
    h->sim->setCPUOperation(true);
    h->sim->setReproducible(true);
    h->active->noise.setReproducibleSeed(seed);
    h->active->setMu(mu);
    h->active->setV0(v0);
    h->active->setEta(eta);
    h->active->setTau(tau);
}
void ref_get_directors(ref_handle* h, double* out) {
    ArrayHandle<dVec> a(h->model->returnDirectors(), access_location::host, access_mode::read);
    for (int i = 0; i < h->model->getNumberOfParticles(); ++i)
        for (int d = 0; d < 3; ++d) out[3 * i + d] = a.data[i].x[d];
}

// dynamicalFeatures(initial, sphere, fraction).computeMSD / computeOverlapFunction
// (src/analysis/dynamicalFeatures.cpp:6-53) on caller positions.
void ref_dynamics(const double* init, const double* cur, int n, double fraction, double radius, double cutoff,
                  double* msd, double* overlap) {
    GPUArray<dVec> a((unsigned int)n, true), b((unsigned int)n, true);
    {
        ArrayHandle<dVec> ha(a, access_location::host, access_mode::overwrite);
        ArrayHandle<dVec> hb(b, access_location::host, access_mode::overwrite);
        for (int i = 0; i < n; ++i)
            for (int d = 0; d < 3; ++d) { ha.data[i].x[d] = init[3 * i + d]; hb.data[i].x[d] = cur[3 * i + d]; }
    }
    dynamicalFeatures df(a, std::make_shared<sphericalDomain>(radius), fraction);
    *msd = df.computeMSD(b);
    *overlap = df.computeOverlapFunction(b, cutoff);
}

// The first `count` save steps of logSpacedIntegers(firstSave, exponent) (inc/simpleUtilities.h:5-41).
void ref_log_spaced(int firstSave, double exponent, int count, long* out) {
    logSpacedIntegers lsi(firstSave, exponent);
    for (int i = 0; i < count; ++i) { out[i] = lsi.nextSave; lsi.update(); }
}

// minimization.cpp:251-262
void ref_fire_setup(ref_handle* h, double dt, double alphaStart, double dtMax, double dtInc, double dtDec,
                    double alphaDec, int nMin, double forceCutoff, double alphaMin, int maxIt) {
    h->fire = std::make_shared<energyMinimizerFIRE>(h->model);
    h->sim = std::make_shared<Simulation>();
    h->sim->setConfiguration(h->model);
    h->fire->setMaximumIterations(maxIt);
    h->fire->setFIREParameters(dt, alphaStart, dtMax, dtInc, dtDec, alphaDec, nMin, forceCutoff, alphaMin);
    h->sim->addUpdater(h->fire, h->model);
    h->sim->setCPUOperation(true);
}
int ref_fire_iterations(ref_handle* h) { return h->fire->getCurrentIterations(); }
void ref_fire_set_max_iterations(ref_handle* h, int n) { h->fire->setMaximumIterations(n); }
double ref_fire_force(ref_handle* h) { return h->fire->getMaxForce(); }

void ref_steps(ref_handle* h, int n) { for (int i = 0; i < n; ++i) h->sim->performTimestep(); }
void ref_set_restricted(ref_handle* h, int r) { h->model->restrictedMotion = r != 0; }
void ref_set_preferred(ref_handle* h, double a0, double p0) { h->model->setPreferredParameters(a0, p0); }
void ref_compute_forces(ref_handle* h) { h->model->computeForces(true); }
void ref_compute_geometry(ref_handle* h) { h->model->computeGeometry(); }
double ref_energy(ref_handle* h) { return h->model->computeEnergy(); }

int ref_num_cells(ref_handle* h) { return h->model->nCells; }
int ref_num_vertices(ref_handle* h) { return h->model->getNumberOfParticles(); }
int ref_ring_width(ref_handle* h) { return (int)h->model->cellNeighborIndex.getW(); }
double ref_radius(ref_handle* h) { return h->model->sphere->radius; }

static void getVec(GPUArray<dVec>& a, double* out, int n) {
    ArrayHandle<dVec> p(a, access_location::host, access_mode::read);
    for (int i = 0; i < n; ++i) for (int d = 0; d < 3; ++d) out[3 * i + d] = p.data[i].x[d];
}
void ref_get_positions(ref_handle* h, double* out) { getVec(h->model->returnPositions(), out, ref_num_vertices(h)); }
void ref_set_positions(ref_handle* h, const double* in) {
    ArrayHandle<dVec> p(h->model->returnPositions(), access_location::host, access_mode::readwrite);
    for (int i = 0; i < ref_num_vertices(h); ++i) for (int d = 0; d < 3; ++d) p.data[i].x[d] = in[3 * i + d];
}
void ref_get_forces(ref_handle* h, double* out) { getVec(h->model->returnForces(), out, ref_num_vertices(h)); }
void ref_get_velocities(ref_handle* h, double* out) { getVec(h->model->returnVelocities(), out, ref_num_vertices(h)); }
void ref_get_cell_positions(ref_handle* h, double* out) { getVec(h->model->cellPositions, out, h->model->nCells); }
void ref_get_area_perimeter(ref_handle* h, double* out) {
    ArrayHandle<scalar2> ap(h->model->areaPerimeter, access_location::host, access_mode::read);
    for (int c = 0; c < h->model->nCells; ++c) { out[2 * c] = ap.data[c].x; out[2 * c + 1] = ap.data[c].y; }
}
// Rings in width Wout (-1 padded) plus counts.
int ref_get_rings(ref_handle* h, int* out, int Wout, unsigned* counts) {
    ArrayHandle<int> cv(h->model->cellNeighbors, access_location::host, access_mode::read);
    ArrayHandle<unsigned int> cn(h->model->cellNumberOfNeighbors, access_location::host, access_mode::read);
    Index2D idx = h->model->cellNeighborIndex;
    for (int c = 0; c < h->model->nCells; ++c) {
        int n = (int)cn.data[c];
        if (n > Wout) return -1;
        counts[c] = (unsigned)n;
        for (int k = 0; k < Wout; ++k) out[(size_t)c * Wout + k] = k < n ? cv.data[idx(k, c)] : -1;
    }
    return 0;
}
void ref_get_vertex_cells(ref_handle* h, int* out) {
    ArrayHandle<int> a(h->model->vertexCellNeighbors, access_location::host, access_mode::read);
    std::memcpy(out, a.data, sizeof(int) * 3 * ref_num_vertices(h));
}
void ref_get_vertex_neighbors(ref_handle* h, int* out) {
    ArrayHandle<int> a(h->model->neighbors, access_location::host, access_mode::read);
    std::memcpy(out, a.data, sizeof(int) * 3 * ref_num_vertices(h));
}

// hyperrectangularCellList over the vertex positions with the parameters the spherical model
// gives its neighbour list: cell size 1.0, radius R + 2.5 (sphericalModel.cpp:21,
// neighborList.cpp:7-20).  Returns Nmax; fills per-bin counts [nside^3] and the slot table.
int ref_cell_list(ref_handle* h, int* nsideOut, unsigned* counts, int* idx, long idxCapacity) {
    double R = h->model->sphere->radius;
    hyperrectangularCellList cl(1.0, R + 2.5);
    cl.computeCellList(h->model->returnPositions());
    iVec ns = cl.getBinsPerSide();
    *nsideOut = ns.x[0];
    int total = cl.totalCells;
    int Nmax = cl.getNmax();
    ArrayHandle<unsigned int> e(cl.elementsPerCell, access_location::host, access_mode::read);
    ArrayHandle<int> pi(cl.particleIndices, access_location::host, access_mode::read);
    if ((long)total * Nmax > idxCapacity) return -1;
    for (int b = 0; b < total; ++b) {
        counts[b] = e.data[b];
        for (int s = 0; s < Nmax; ++s)
            idx[(long)b * Nmax + s] = s < (int)e.data[b] ? pi.data[cl.cellListIndexer(s, b)] : -1;
    }
    return Nmax;
}

// neighborList(range, radius, subGrid).computeNeighborLists over caller points (neighborList.cpp:
// 7-20, 96-151, CPU branch).  Returns Nmax, or -Nmax when `capacity` (entries) is too small.
int ref_neighbor_list(const double* pts, int np, double range, double radius, int subGrid, unsigned* npp, int* idx,
                      double* vec, double* dist, long capacity) {
    GPUArray<dVec> points((unsigned int)np, true);
    {
        ArrayHandle<dVec> p(points, access_location::host, access_mode::overwrite);
        for (int i = 0; i < np; ++i)
            for (int d = 0; d < 3; ++d) p.data[i].x[d] = pts[3 * i + d];
    }
    neighborList nl(range, radius, subGrid);
    nl.computeNeighborLists(points);
    const int Nmax = nl.Nmax;
    if ((long)np * Nmax > capacity) return -Nmax;
    ArrayHandle<unsigned int> hn(nl.neighborsPerParticle, access_location::host, access_mode::read);
    ArrayHandle<int> hi(nl.particleIndices, access_location::host, access_mode::read);
    ArrayHandle<dVec> hv(nl.neighborVectors, access_location::host, access_mode::read);
    ArrayHandle<scalar> hd(nl.neighborDistances, access_location::host, access_mode::read);
    for (int pp = 0; pp < np; ++pp) {
        npp[pp] = hn.data[pp];
        for (int k = 0; k < Nmax; ++k) {
            const int at = nl.neighborIndexer(k, pp);
            const long o = (long)pp * Nmax + k;
            idx[o] = hi.data[at];
            dist[o] = hd.data[at];
            for (int d = 0; d < 3; ++d) vec[3 * o + d] = hv.data[at].x[d];
        }
    }
    return Nmax;
}

}  // extern "C"
