// C++ host classes over the libsvm C ABI, with the class and method names of the reference
// (src/model/sphericalVertexModel.h, src/updaters/brownianDynamics.h,
// src/updaters/energyMinimizerFIRE.h, src/simulation/simulation.h), so a driver written
// against the reference compiles against this header with its includes swapped.  The state
// lives on the GPU; there is no CPU branch (setCPUOperation(true) throws).  Failures of the C ABI
// are raised as std::runtime_error, as the reference's HANDLE_ERROR raises (inc/std_include.h:123-134).
#pragma once
#include <cmath>
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
        check(svm_topology_from_points(centres.data(), n, &t), "svm_topology_from_points");
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
        computeGeometry();
    }

    // parameters
    void setPreferredParameters(scalar a0, scalar p0) { check(svm_model_set_preferred_parameters(h(), a0, p0), "setPreferredParameters"); }
    void setScalarModelParameter(scalar kr) { Kr = kr; check(svm_model_set_scalar_model_parameter(h(), kr), "setScalarModelParameter"); }
    void setT1Threshold(scalar t) { t1Threshold = t; check(svm_model_set_t1_threshold(h(), t), "setT1Threshold"); }
    void setRestrictedMotion(bool r) { restrictedMotion = r; check(svm_model_set_restricted_motion(h(), r), "restrictedMotion"); }
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

  private:
    struct Del { void operator()(svm_model* p) const { svm_model_destroy(p); } };
    std::unique_ptr<svm_model, Del> m;
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
    void setMaximumIterations(int n) { maxIterations = n; reset(); }
    void performUpdate() override { minimize(); }
    void minimize() {
        ensure();
        int it = 0;
        double v = 0;
        check(svm_fire_minimize(f, criterion, &it, &v), "minimize");
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
