// C++ host classes over the libsvm C ABI, with the class and method names of the reference
// (src/model/sphericalVertexModel.h, src/updaters/brownianDynamics.h,
// src/updaters/energyMinimizerFIRE.h, src/simulation/simulation.h), so a driver written
// against the reference compiles against this header with its includes swapped.  The state
// lives on the GPU; there is no CPU branch (setCPUOperation(true) throws).  Failures of the C ABI
// are raised as std::runtime_error, as the reference's HANDLE_ERROR raises (inc/std_include.h:123-134).
#pragma once
#include <algorithm>
#include <cmath>
#include <iostream>
#include <array>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "svm.h"

namespace svmgpu {

inline void check(int rc, const char* what) {
    if (rc != SVM_OK) throw std::runtime_error(std::string(what) + ": " + svm_status_string(rc));
}

using scalar = double;

// noiseSource (src/utilities/noiseSource.h:17-76): the reproducible seed of the initial cell
// centres and of the in-kernel noise stream.
class noiseSource {
  public:
    explicit noiseSource(bool rep = false) : Reproducible(rep) {}
    void setReproducibleSeed(int seed) { RNGSeed = seed; Reproducible = true; }
    void setReproducible(bool rep) { Reproducible = rep; }
    bool Reproducible;
    int RNGSeed = -1;
};

// a created model and its sizes (used by derived models that build their own handle)
struct ModelHandle {
    svm_model* h;
    int nCells, nVertices, ringCapacity;
};

// sphericalVertexModel (src/model/sphericalVertexModel.h:10-123); n counts cells.
class sphericalVertexModel {
  public:
    sphericalVertexModel(int n, noiseSource& noise, scalar a0 = 1.0, scalar p0 = 3.8, bool useGPU = true,
                         bool neverGPU = false, int ringCapacity = 16)
        : nCells(n) {
        if (!useGPU || neverGPU) throw std::runtime_error("this model runs on the GPU only");
        std::vector<double> centres(3 * (size_t)n);
        check(svm_random_cell_centres(noise.RNGSeed, n, centres.data()), "svm_random_cell_centres");
        svm_topology* t = nullptr;
        check(svm_topology_from_points_gpu(centres.data(), n, nullptr, &t), "svm_topology_from_points_gpu");
        int nc = 0, nv = 0, maxRing = 0;
        svm_topology_sizes(t, &nc, &nv, &maxRing);
        nVertices = nv;
        std::vector<double> vp(3 * (size_t)nv);
        std::vector<int> rings((size_t)n * maxRing), vc(3 * (size_t)nv), vn(3 * (size_t)nv);
        std::vector<unsigned> counts(n);
        int rc = svm_topology_get(t, vp.data(), rings.data(), maxRing, counts.data(), vc.data(), vn.data());
        svm_topology_free(t);
        check(rc, "svm_topology_get");
        ringCapacity = std::max(ringCapacity, maxRing + 1);
        radius = std::sqrt(n / (4.0 * M_PI));
        svm_model* h = nullptr;
        check(svm_model_create(n, nv, ringCapacity, radius, nullptr, &h), "svm_model_create");
        m.reset(h);
        check(svm_model_set_topology(h, vp.data(), rings.data(), maxRing, counts.data(), vc.data(), vn.data()),
              "svm_model_set_topology");
        setT1Threshold(0.1);  // sphericalVertexModel.cpp:13
        setPreferredParameters(a0, p0);
        setScalarModelParameter(1.0);
        std::vector<double> dirs(3 * (size_t)nv);  // made as sphericalVertexModel.cpp:58-70, seeded
        check(svm_random_vertex_directors(noise.RNGSeed, n, vp.data(), nv, dirs.data()), "svm_random_vertex_directors");
        check(svm_model_set_directors(h, dirs.data()), "svm_model_set_directors");
        computeGeometry();
    }

    // parameters
    void setPreferredParameters(scalar a0, scalar p0) { check(svm_model_set_preferred_parameters(h(), a0, p0), "setPreferredParameters"); }
    void setScalarModelParameter(scalar kr) { Kr = kr; check(svm_model_set_scalar_model_parameter(h(), kr), "setScalarModelParameter"); }
    void setT1Threshold(scalar t) { t1Threshold = t; check(svm_model_set_t1_threshold(h(), t), "setT1Threshold"); }
    void setRestrictedMotion(bool r) { restrictedMotion = r; check(svm_model_set_restricted_motion(h(), r), "restrictedMotion"); }
    // SVM_PRECISION_FP64 (the plain form), SVM_PRECISION_MIXED (FP32 bulk, FP64 areas/energy/
    // renormalisation) or SVM_PRECISION_FP64_VECTOR (FP64 with the vector-form gradient)
    void setPrecision(int precision) { check(svm_model_set_precision(h(), precision), "setPrecision"); }
    int getNumberOfParticles() const { return nVertices; }

    // the path
    void computeGeometry() { check(svm_model_compute_geometry(h()), "computeGeometry"); }
    void computeForces(bool = true) { check(svm_model_compute_forces(h()), "computeForces"); }
    scalar computeEnergy() { double e = 0; check(svm_model_compute_energy(h(), &e), "computeEnergy"); return e; }
    void moveParticles(const std::vector<double>& disp, scalar scale = 1.) {
        check(svm_model_move_particles_host(h(), disp.data(), scale), "moveParticles");
    }
    void enforceTopology() { check(svm_model_enforce_topology(h()), "enforceTopology"); }

    // state
    std::vector<double> returnPositions() { std::vector<double> p(3 * (size_t)nVertices); check(svm_model_get_positions(h(), p.data()), "positions"); return p; }
    std::vector<double> returnForces() { std::vector<double> p(3 * (size_t)nVertices); check(svm_model_get_forces(h(), p.data()), "forces"); return p; }
    std::vector<double> areaPerimeter() { std::vector<double> p(2 * (size_t)nCells); check(svm_model_get_area_perimeter(h(), p.data()), "areaPerimeter"); return p; }

    svm_model* h() const { return m.get(); }

    int nCells, nVertices = 0, ringCapacity = 16;
    scalar radius = 1.0, Kr = 1.0, t1Threshold = 0.1;
    bool restrictedMotion = false;

  protected:
    // adopts an already created model (batches)
    explicit sphericalVertexModel(ModelHandle mh)
        : nCells(mh.nCells), nVertices(mh.nVertices), ringCapacity(mh.ringCapacity), m(mh.h) {}

  private:
    struct Del { void operator()(svm_model* p) const { svm_model_destroy(p); } };
    std::unique_ptr<svm_model, Del> m;
};

// Independent spheres of uneven size in one model (svm_batch_* in svm.h; no counterpart in the
// reference, which runs one sphere per process).  Replica r has nCellsPerReplica[r] cells from
// the seeded recipe with seeds[r] and radius sqrt(N_r / 4 pi); the batch runs the mixed form, and a
// brownianDynamics updater drives it with the per-replica temperatures of setTemperatures.
namespace detail {
// concatenated topology of a batch, built before the model base class is constructed
struct BatchTopo {
    std::vector<double> vp;
    std::vector<int> rings, vc, vn;
    std::vector<unsigned> counts;
    int nv = 0, cap = 0;
};
struct BatchTopoHolder {
    BatchTopo topo;
};
}  // namespace detail

class sphericalVertexModelBatch : private detail::BatchTopoHolder, public sphericalVertexModel {
  public:
    sphericalVertexModelBatch(const std::vector<int>& nCellsPerReplica, const std::vector<int>& seeds, scalar a0 = 1.0,
                              scalar p0 = 3.8, int cap = 16)
        : sphericalVertexModel(create(nCellsPerReplica, seeds, cap, topo)) {
        nReplicas = (int)nCellsPerReplica.size();
        check(svm_model_set_topology(h(), topo.vp.data(), topo.rings.data(), topo.cap, topo.counts.data(), topo.vc.data(),
                                     topo.vn.data()),
              "svm_model_set_topology");
        topo = detail::BatchTopo{};
        setT1Threshold(0.1);
        setPreferredParameters(a0, p0);
        setScalarModelParameter(1.0);
        computeGeometry();
    }
    void setTemperatures(const std::vector<double>& T) { check(svm_batch_set_temperatures(h(), T.data()), "setTemperatures"); }
    std::vector<double> replicaEnergies() {
        std::vector<double> e(nReplicas);
        check(svm_batch_energies(h(), e.data()), "replicaEnergies");
        return e;
    }
    // kernelTuner-style block-size tuning of the batch kernels (lo <= 0: off)
    void autotune(int lo = 64, int hi = 1024, int step = 64, int nSamples = 3, int period = 1000) {
        check(svm_batch_autotune(h(), lo, hi, step, nSamples, period), "autotune");
    }
    int nReplicas = 0;

  private:
    using Topo = detail::BatchTopo;
    static ModelHandle create(const std::vector<int>& n, const std::vector<int>& seeds, int cap, Topo& T) {
        if (n.size() != seeds.size() || n.empty()) throw std::runtime_error("one seed per replica");
        struct One { std::vector<double> vp; std::vector<int> rings, vc, vn; std::vector<unsigned> counts; int nv, w; };
        std::vector<One> reps;
        std::vector<int> nvs;
        std::vector<double> radius;
        int width = cap;
        for (size_t r = 0; r < n.size(); ++r) {
            std::vector<double> centres(3 * (size_t)n[r]);
            check(svm_random_cell_centres(seeds[r], n[r], centres.data()), "svm_random_cell_centres");
            svm_topology* t = nullptr;
            check(svm_topology_from_points_gpu(centres.data(), n[r], nullptr, &t), "svm_topology_from_points_gpu");
            int nc = 0, nv = 0, mr = 0;
            svm_topology_sizes(t, &nc, &nv, &mr);
            One o{std::vector<double>(3 * (size_t)nv), std::vector<int>((size_t)nc * mr), std::vector<int>(3 * (size_t)nv),
                  std::vector<int>(3 * (size_t)nv), std::vector<unsigned>(nc), nv, mr};
            const int rc = svm_topology_get(t, o.vp.data(), o.rings.data(), mr, o.counts.data(), o.vc.data(), o.vn.data());
            svm_topology_free(t);
            check(rc, "svm_topology_get");
            width = std::max(width, mr + 1);
            nvs.push_back(nv);
            radius.push_back(std::sqrt(n[r] / (4.0 * M_PI)));
            reps.push_back(std::move(o));
        }
        int cOff = 0, vOff = 0;
        T.cap = width;
        for (size_t r = 0; r < reps.size(); ++r) {
            const One& o = reps[r];
            for (double x : o.vp) T.vp.push_back(x);
            for (int c = 0; c < n[r]; ++c) {
                for (int k = 0; k < width; ++k)
                    T.rings.push_back(k < o.w && o.rings[(size_t)c * o.w + k] >= 0 ? o.rings[(size_t)c * o.w + k] + vOff : -1);
                T.counts.push_back(o.counts[c]);
            }
            for (int x : o.vc) T.vc.push_back(x + cOff);
            for (int x : o.vn) T.vn.push_back(x + vOff);
            cOff += n[r];
            vOff += o.nv;
        }
        T.nv = vOff;
        svm_model* h = nullptr;
        check(svm_batch_create((int)n.size(), n.data(), nvs.data(), width, radius.data(), nullptr, &h), "svm_batch_create");
        return ModelHandle{h, cOff, vOff, width};
    }
};

// kernelTuner (src/utilities/kernelTuner.{h,cpp}): bracket a launch with begin()/end() and launch
// with getParameter(); CUDA events on `stream` (nullptr: the legacy default stream).
class kernelTuner {
  public:
    kernelTuner(int start, int end, int step, int nSamples, int period, void* stream = nullptr) {
        check(svm_tuner_create(start, end, step, nSamples, period, stream, &t), "kernelTuner");
    }
    ~kernelTuner() { svm_tuner_destroy(t); }
    kernelTuner(const kernelTuner&) = delete;
    kernelTuner& operator=(const kernelTuner&) = delete;
    void begin() { check(svm_tuner_begin(t), "kernelTuner::begin"); }
    void end() { check(svm_tuner_end(t), "kernelTuner::end"); }
    int getParameter() { int v = 0; check(svm_tuner_parameter(t, &v), "kernelTuner::getParameter"); return v; }
    bool samplingComplete() { int d = 0; check(svm_tuner_sampling_complete(t, &d), "samplingComplete"); return d != 0; }
    void printTimingData() {
        int n = 0;
        svm_tuner_timing_data(t, nullptr, nullptr, 0, &n);
        std::vector<int> c(n);
        std::vector<float> med(n);
        svm_tuner_timing_data(t, c.data(), med.data(), n, &n);
        std::cout << "parameter used: " << getParameter() << std::endl;
        for (int i = 1; i < n; ++i) std::cout << "tuner value " << c[i] << " median time " << med[i] << std::endl;
    }

  private:
    svm_tuner* t = nullptr;
};

class updater {
  public:
    virtual ~updater() = default;
    virtual void performUpdate() = 0;
    virtual void setModel(std::shared_ptr<sphericalVertexModel> mdl) { model = std::move(mdl); }
    virtual void setDeltaT(scalar dt) { deltaT = dt; }
    virtual void setReproducible(bool r) { reproducible = r; }
    std::shared_ptr<sphericalVertexModel> model;
    scalar deltaT = 0.01;
    bool reproducible = true;
};

// brownianDynamics (src/updaters/brownianDynamics.h:11-29)
class brownianDynamics : public updater {
  public:
    explicit brownianDynamics(bool rep = true) { reproducible = rep; noise.setReproducible(rep); }
    void setT(scalar t) { temperature = t; }
    void performUpdate() override { integrateEquationOfMotion(); }
    void integrateEquationOfMotion() {
        const uint64_t seed = noise.RNGSeed >= 0 ? (uint64_t)noise.RNGSeed : 1337u;
        check(svm_brownian_step(model->h(), temperature, deltaT, mu, SVM_NOISE_PHILOX, nullptr, seed), "brownian step");
    }
    scalar temperature = 0.0, mu = 1.0;
    noiseSource noise;
};

// sphericalSelfPropelledParticle (src/updaters/sphericalSelfPropelledParticle.h:13-25, with the
// parameters of vectorialVicsek.h:31-44)
class sphericalSelfPropelledParticle : public updater {
  public:
    explicit sphericalSelfPropelledParticle(bool rep = true) { reproducible = rep; noise.setReproducible(rep); }
    void setMu(scalar m) { mu = m; }
    void setV0(scalar v) { v0 = v; }
    void setTau(scalar t) { tau = t; }
    void performUpdate() override { integrateEquationOfMotion(); }
    void integrateEquationOfMotion() {
        const uint64_t seed = noise.RNGSeed >= 0 ? (uint64_t)noise.RNGSeed : 1337u;
        check(svm_spp_step(model->h(), deltaT, mu, v0, tau, SVM_NOISE_PHILOX, nullptr, seed), "spp step");
    }
    scalar mu = 1.0, v0 = 0.0, tau = 1.0;
    noiseSource noise;
};

// sphericalVectorialVicsek (src/updaters/sphericalVectorialVicsek.{h,cpp}; defaults of
// vectorialVicsek.h:11): the self-propelled move, then each director relaxes at rate dt / tau towards
// the tangent average of itself and its three vertex neighbours plus Eta times a random tangent
// unit vector.
class sphericalVectorialVicsek : public updater {
  public:
    explicit sphericalVectorialVicsek(bool rep = true) { reproducible = rep; noise.setReproducible(rep); }
    void setMu(scalar m) { mu = m; }
    void setV0(scalar v) { v0 = v; }
    void setEta(scalar e) { Eta = e; }
    void setTau(scalar t) { tau = t; }
    void performUpdate() override { integrateEquationOfMotion(); }
    void integrateEquationOfMotion() {
        const uint64_t seed = noise.RNGSeed >= 0 ? (uint64_t)noise.RNGSeed : 1337u;
        check(svm_vicsek_step(model->h(), deltaT, mu, v0, Eta, tau, SVM_NOISE_PHILOX, nullptr, seed), "vicsek step");
    }
    scalar mu = 1.0, v0 = 0.01, Eta = 1.0, tau = 1.0;
    noiseSource noise;
};

// neighborList (src/utilities/neighborList.h:8-75): metric neighbours within maxRange of each point
// (minimum image in a periodic box of side 2 radius), rows of Nmax entries, zero past each count.
class neighborList {
  public:
    neighborList(scalar range, scalar sphereRadius, int subGridReduction = 1, int slotCapacity = 16)
        : maxRange(range), radius(sphereRadius), sub(subGridReduction), cap(slotCapacity) {}
    ~neighborList() { if (nl) svm_neighbor_list_destroy(nl); }
    neighborList(const neighborList&) = delete;
    neighborList& operator=(const neighborList&) = delete;
    // the model's current vertex positions
    void computeNeighborLists(sphericalVertexModel& m) {
        ensure(m.getNumberOfParticles());
        check(svm_neighbor_list_compute_model(nl, m.h()), "computeNeighborLists");
        fetch();
    }
    // caller points already on the device (AoS double[3 n])
    void computeNeighborLists(const double* pointsDevice, int n) {
        ensure(n);
        check(svm_neighbor_list_compute(nl, pointsDevice, n), "computeNeighborLists");
        fetch();
    }
    scalar maxRange, radius;
    int Nmax = 4;
    std::vector<unsigned> neighborsPerParticle;
    std::vector<int> particleIndices;       // [n * Nmax], row per point
    std::vector<double> neighborVectors;    // [n * Nmax * 3]
    std::vector<double> neighborDistances;  // [n * Nmax]

  private:
    void ensure(int n) {
        if (nl && n == nPoints) return;
        if (nl) svm_neighbor_list_destroy(nl);
        nl = nullptr;
        check(svm_neighbor_list_create(maxRange, radius, sub, n, cap, nullptr, &nl), "neighborList");
        nPoints = n;
    }
    void fetch() {
        check(svm_neighbor_list_get(nl, &Nmax, nullptr, nullptr, nullptr, nullptr, 0), "get");
        const size_t e = (size_t)nPoints * Nmax;
        neighborsPerParticle.resize(nPoints);
        particleIndices.resize(e);
        neighborVectors.resize(3 * e);
        neighborDistances.resize(e);
        check(svm_neighbor_list_get(nl, &Nmax, neighborsPerParticle.data(), particleIndices.data(),
                                    neighborVectors.data(), neighborDistances.data(), (long)e), "get");
    }
    int sub, cap, nPoints = 0;
    svm_neighbor_list* nl = nullptr;
};

// velocityVerlet (src/updaters/velocityVerlet.{h,cpp}), unit masses: per step the displacement
// dt v + dt^2/2 F with the first half kick, the move (T1 flips unless motion is restricted),
// geometry and forces, the second half kick.  Forces must be current before the first step.
class velocityVerlet : public updater {
  public:
    void performUpdate() override { integrateEquationOfMotion(); }
    void integrateEquationOfMotion() { check(svm_velocity_verlet_step(model->h(), deltaT, 1), "velocity Verlet"); }
    // gpu_update_velocity (velocityVerlet.cuh:14-19): v += dt/2 F
    void updateVelocity() { check(svm_vv_half(model->h(), deltaT), "velocity half kick"); }
};

// gpu_dVec_dot_products (src/utilities/utilities.cuh:74) over the model's forces and velocities:
// {sum F.v, sum F.F, sum v.v, max |F|}
inline std::array<double, 4> dotProducts(sphericalVertexModel& m) {
    std::array<double, 4> out{};
    check(svm_reduce_dots(m.h(), out.data()), "dot products");
    return out;
}

// energyMinimizerFIRE (src/updaters/energyMinimizerFIRE.h:27-68)
class energyMinimizerFIRE : public updater {
  public:
    explicit energyMinimizerFIRE(std::shared_ptr<sphericalVertexModel> mdl) { setModel(std::move(mdl)); }
    ~energyMinimizerFIRE() override { if (f) svm_fire_destroy(f); }
    void setFIREParameters(scalar dt, scalar alphaStart, scalar dtMax, scalar dtInc, scalar dtDec, scalar alphaDec,
                           int nMin, scalar forceCutoff, scalar alphaMin = 0.75) {
        p = {dt, alphaStart, dtMax, dtInc, dtDec, alphaDec, (double)nMin, forceCutoff, alphaMin};
        reset();
    }
    void setMaximumIterations(int n) {
        maxIterations = n;
        if (f) check(svm_fire_set_max_iterations(f, n), "setMaximumIterations");
    }
    void performUpdate() override { minimize(); }
    void minimize() {
        ensure();
        int it = 0;
        double v = 0;
        check(svm_fire_minimize(f, criterion, &it, &v), "minimize");
    }
    // fireStep (energyMinimizerFIRE.h:56): sums, velocity update and dt/alpha control on the current
    // forces and velocities; integrateEquationOfMotion is the velocity-Verlet step at the current dt
    void fireStep() { ensure(); check(svm_fire_step(f), "fireStep"); }
    void integrateEquationOfMotion() {
        double s[7];
        ensure();
        check(svm_fire_state(f, s), "state");
        check(svm_velocity_verlet_step(model->h(), s[0], 1), "velocity Verlet");
    }
    scalar getMaxForce() { double s[7]; ensure(); check(svm_fire_state(f, s), "state"); return s[3]; }
    int getCurrentIterations() { double s[7]; ensure(); check(svm_fire_state(f, s), "state"); return (int)s[6]; }
    int criterion = SVM_FIRE_RMS_OVER_N;

  private:
    void reset() { if (f) { svm_fire_destroy(f); f = nullptr; } }
    void ensure() {
        if (!f)
            check(svm_fire_create(model->h(), p[0], p[1], p[2], p[3], p[4], p[5], (int)p[6], p[7], p[8], maxIterations, &f),
                  "svm_fire_create");
    }
    // initializeParameters defaults (energyMinimizerFIRE.cpp:22-41)
    std::vector<double> p{0.01, 0.99, 0.1, 1.05, 0.95, 0.9, 5, 1e-7, 0.0};
    int maxIterations = 1000;
    svm_fire* f = nullptr;
};

// Simulation (src/simulation/simulation.{h,cpp})
class Simulation {
  public:
    void setConfiguration(std::shared_ptr<sphericalVertexModel> c) { configuration = std::move(c); }
    void addUpdater(std::shared_ptr<updater> u, std::shared_ptr<sphericalVertexModel> c) {
        u->setModel(std::move(c));
        updaters.push_back(std::move(u));
    }
    void setIntegrationTimestep(scalar dt) { integrationTimestep = dt; for (auto& u : updaters) u->setDeltaT(dt); }
    void setCPUOperation(bool setcpu) { if (setcpu) throw std::runtime_error("CPU operation is not available"); }
    void setReproducible(bool r) { for (auto& u : updaters) u->setReproducible(r); }
    void computeForces() { configuration->computeForces(true); }
    scalar computeEnergy() { return configuration->computeEnergy(); }
    void performTimestep() {
        integerTimestep += 1;
        Time += integrationTimestep;
        for (auto& u : updaters) u->performUpdate();
    }
    std::shared_ptr<sphericalVertexModel> configuration;
    std::vector<std::shared_ptr<updater>> updaters;
    int integerTimestep = 0;
    scalar Time = 0.0, integrationTimestep = 0.01;
};

}  // namespace svmgpu
