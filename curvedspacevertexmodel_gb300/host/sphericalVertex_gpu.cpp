// The reference's Brownian driver (sphericalVertex.cpp:86-138) written against svm.hpp:
// build a model from a seed, equilibrate at T = 0 with p0 = 1, then run at (T, p0), printing the
// energy and the timing.  Usage: sphericalVertex_gpu [N cells] [iterations] [T] [p0] [dt] [seed]
//
// With "batch" as the first argument it runs replicas of sizes N, 2N, 3N (seeds seed, seed+1,
// seed+2; temperatures T, 2T, 3T) as one sphericalVertexModelBatch and prints each replica's
// energy:  sphericalVertex_gpu batch [N] [iterations] [T] [p0] [dt] [seed]
//
// With "fire" it relaxes a stabilised model by FIRE driven phase by phase, as minimize does
// (velocityVerlet step at the minimizer's dt, then fireStep), and prints the energy and the dot
// products:  sphericalVertex_gpu fire [N] [iterations] [seed]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

#include "svm.hpp"

using namespace svmgpu;

static int run_batch(int argc, char** argv) {
    const int N = argc > 2 ? std::atoi(argv[2]) : 200;
    const int iterations = argc > 3 ? std::atoi(argv[3]) : 100;
    const double T = argc > 4 ? std::atof(argv[4]) : 0.01;
    const double p0 = argc > 5 ? std::atof(argv[5]) : 3.8;
    const double dt = argc > 6 ? std::atof(argv[6]) : 0.01;
    const int seed = argc > 7 ? std::atoi(argv[7]) : 1137;
    try {
        auto batch = std::make_shared<sphericalVertexModelBatch>(std::vector<int>{N, 2 * N, 3 * N},
                                                                 std::vector<int>{seed, seed + 1, seed + 2}, 1.0, p0);
        batch->setT1Threshold(0.04);
        auto BD = std::make_shared<brownianDynamics>(true);
        BD->noise.setReproducibleSeed(seed + 7);
        BD->setModel(batch);
        BD->setDeltaT(dt);
        batch->setTemperatures({T, 2 * T, 3 * T});
        for (int i = 0; i < iterations; ++i) BD->performUpdate();
        batch->computeGeometry();
        const std::vector<double> e = batch->replicaEnergies();
        std::printf("{\"replicas\": %d, \"vertices\": %d, \"energies\": [%.17g, %.17g, %.17g]}\n", batch->nReplicas,
                    batch->getNumberOfParticles(), e[0], e[1], e[2]);
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 1;
    }
    return 0;
}

// "active N steps seed": the Vicsek updater on the model through the C++ classes, then the model's
// neighbour list (range 1, radius R + 2.5, as sphericalModel.cpp:21 sets it up).
static int run_active(int argc, char** argv) {
    const int N = argc > 2 ? std::atoi(argv[2]) : 200;
    const int iterations = argc > 3 ? std::atoi(argv[3]) : 100;
    const int seed = argc > 4 ? std::atoi(argv[4]) : 1137;
    try {
        noiseSource noise(true);
        noise.setReproducibleSeed(seed);
        auto model = std::make_shared<sphericalVertexModel>(N, noise, 1.0, 3.8, true, false);
        model->setT1Threshold(0.04);
        auto V = std::make_shared<sphericalVectorialVicsek>(true);
        V->noise.setReproducibleSeed(seed + 3);
        V->setModel(model);
        V->setDeltaT(0.01);
        V->setV0(0.1);
        V->setEta(0.4);
        V->setTau(0.5);
        for (int i = 0; i < iterations; ++i) V->performUpdate();
        model->computeGeometry();
        const double e = model->computeEnergy();
        neighborList nl(1.0, model->radius + 2.5);
        nl.computeNeighborLists(*model);
        long pairs = 0, indexSum = 0;
        for (unsigned c : nl.neighborsPerParticle) pairs += c;
        for (int j : nl.particleIndices) indexSum += j;
        std::printf("{\"vertices\": %d, \"energy\": %.17g, \"Nmax\": %d, \"pairs\": %ld, \"index_sum\": %ld}\n",
                    model->getNumberOfParticles(), e, nl.Nmax, pairs, indexSum);
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 1;
    }
    return 0;
}

// "fire N iterations seed": 50 stabilisation steps (T = 0, p0 = 1), then p0 = 3.8 and FIRE
// (dt 0.01, alpha0 0.1, dtMax 0.1, finc 1.1, fdec 0.5, alphaDec 0.9, NMin 5) driven phase by phase.
static int run_fire(int argc, char** argv) {
    const int N = argc > 2 ? std::atoi(argv[2]) : 200;
    const int iterations = argc > 3 ? std::atoi(argv[3]) : 100;
    const int seed = argc > 4 ? std::atoi(argv[4]) : 1137;
    try {
        noiseSource noise(true);
        noise.setReproducibleSeed(seed);
        auto model = std::make_shared<sphericalVertexModel>(N, noise, 1.0, 1.0, true, false);
        model->setT1Threshold(0.04);
        auto BD = std::make_shared<brownianDynamics>(true);
        BD->noise.setReproducibleSeed(seed + 1);
        BD->setModel(model);
        for (int i = 0; i < 50; ++i) BD->performUpdate();
        model->setPreferredParameters(1.0, 3.8);
        energyMinimizerFIRE fire(model);
        fire.setFIREParameters(0.01, 0.1, 0.1, 1.1, 0.5, 0.9, 5, 1e-300, 0.0);
        fire.setMaximumIterations(iterations);
        model->computeForces();
        for (int i = 0; i < iterations; ++i) {
            fire.integrateEquationOfMotion();
            fire.fireStep();
        }
        const std::array<double, 4> d = dotProducts(*model);
        model->computeGeometry();
        const double e = model->computeEnergy();
        std::printf("{\"vertices\": %d, \"energy\": %.17g, \"dots\": [%.17g, %.17g, %.17g, %.17g]}\n",
                    model->getNumberOfParticles(), e, d[0], d[1], d[2], d[3]);
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 1;
    }
    return 0;
}

int main(int argc, char** argv) {
    if (argc > 1 && std::string(argv[1]) == "batch") return run_batch(argc, argv);
    if (argc > 1 && std::string(argv[1]) == "fire") return run_fire(argc, argv);
    if (argc > 1 && std::string(argv[1]) == "active") return run_active(argc, argv);
    const int N = argc > 1 ? std::atoi(argv[1]) : 200;
    const int iterations = argc > 2 ? std::atoi(argv[2]) : 100;
    const double T = argc > 3 ? std::atof(argv[3]) : 0.01;
    const double p0 = argc > 4 ? std::atof(argv[4]) : 3.8;
    const double dt = argc > 5 ? std::atof(argv[5]) : 0.01;
    const int seed = argc > 6 ? std::atoi(argv[6]) : 1137;
    try {
        noiseSource noise(true);
        noise.setReproducibleSeed(seed);
        auto configuration = std::make_shared<sphericalVertexModel>(N, noise, 1.0, p0, true, false);
        auto BD = std::make_shared<brownianDynamics>(true);
        BD->noise.setReproducibleSeed(seed + 1);
        auto sim = std::make_shared<Simulation>();
        sim->setConfiguration(configuration);
        sim->addUpdater(BD, configuration);
        sim->setIntegrationTimestep(dt);
        sim->setCPUOperation(false);
        sim->setReproducible(true);
        BD->setT(0);
        configuration->setPreferredParameters(1.0, 1.0);
        for (int i = 0; i < iterations; ++i) sim->performTimestep();
        BD->setT(T);
        configuration->setPreferredParameters(1.0, p0);
        auto t0 = std::chrono::steady_clock::now();
        for (int i = 0; i < iterations; ++i) sim->performTimestep();
        configuration->computeGeometry();
        const double e = configuration->computeEnergy();
        auto t1 = std::chrono::steady_clock::now();
        const double s = std::chrono::duration<double>(t1 - t0).count();
        std::printf("{\"cells\": %d, \"vertices\": %d, \"steps\": %d, \"energy\": %.17g, \"seconds\": %.6f}\n", N,
                    configuration->getNumberOfParticles(), iterations, e, s);
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 1;
    }
    return 0;
}
