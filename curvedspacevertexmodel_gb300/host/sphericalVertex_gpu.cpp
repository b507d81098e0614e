// The reference's Brownian driver (sphericalVertex.cpp:86-138) written against svm.hpp:
// build a model from a seed, equilibrate at T = 0 with p0 = 1, then run at (T, p0), printing the
// energy and the timing.  Usage: sphericalVertex_gpu [N cells] [iterations] [T] [p0] [dt] [seed]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <memory>

#include "svm.hpp"

using namespace svmgpu;

int main(int argc, char** argv) {
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
