// NaiveAlgorithm.cpp -- the loop of NaiveAlgorithm::startSimulation (NaiveAlgorithm.cpp:15-260)
// over the C ABI: initial accelerations, then per step leapfrog part 1, accelerations, leapfrog
// part 2, with positions/velocities/|a|/energy captured on visualised steps. All work goes to
// one stream; the host waits only at visualised steps (see nBodyAlgorithm.hpp).
#include "NaiveAlgorithm.hpp"

#include <cmath>
#include <iostream>

NaiveAlgorithm::NaiveAlgorithm(double dt, double tEnd, double vs, std::string& outDir)
    : nBodyAlgorithm(dt, tEnd, vs, outDir) {
    description = "Naive Algorithm";
}

void NaiveAlgorithm::computeAccelerations() {
    nb_throw_if(nb_naive_accel(ctx, d_m, d_x, d_y, d_z, d_ax, d_ay, d_az, n, G,
                               configuration::epsilon2, precisionMode(),
                               configuration::naive_algorithm::blockSize, stream),
                "nb_naive_accel");
}

void NaiveAlgorithm::startSimulation(const SimulationData& d) {
    positions_x[0] = d.positions_x;
    positions_y[0] = d.positions_y;
    positions_z[0] = d.positions_z;
    velocities_x[0] = d.velocities_x;
    velocities_y[0] = d.velocities_y;
    velocities_z[0] = d.velocities_z;
    adjustVelocities(d);
    upload(d);
    timer.setProperties(description, n, deviceName);
    timer.addTimingSequence("Acceleration Kernel Time");
    timer.addTimingSequence("Leapfrog Part 1");
    timer.addTimingSequence("Leapfrog Part 2");

    double time = 0.0, sinceVis = 0.0;
    d_type::int_t step = 0;
    int a0 = phases.mark(stream);
    computeAccelerations();
    phases.span("Acceleration Kernel Time", a0, phases.mark(stream));
    storeAccelerations(step);
    if (configuration::compute_energy) computeEnergy(step);
    finishVisualisedStep(step, d);
    std::cout << "Finished initial step " << step << std::endl << std::endl;
    time += dt;
    sinceVis += dt;
    step += 1;
    while (time <= t_end + 0.000001) {
        const bool vis = std::abs(sinceVis - visualizationStepWidth) < 0.000001;
        const int t0 = phases.mark(stream);
        leapfrogPart1();
        const int t1 = phases.mark(stream);
        if (vis) stagePositions();
        const int t2 = phases.mark(stream);
        computeAccelerations();
        const int t3 = phases.mark(stream);
        leapfrogPart2();
        const int t4 = phases.mark(stream);
        phases.span("Leapfrog Part 1", t0, t1);
        phases.span("Acceleration Kernel Time", t2, t3);
        phases.span("Leapfrog Part 2", t3, t4);
        if (vis) {
            stageVelocitiesAndAccelerations(step);
            finishVisualisedStep(step, d);
            std::cout << "Finished step " << step << std::endl << std::endl;
            step += 1;
            sinceVis = 0.0;
        } else {
            syncIfManyPending();
        }
        time += dt;
        sinceVis += dt;
    }
    sync();
}
