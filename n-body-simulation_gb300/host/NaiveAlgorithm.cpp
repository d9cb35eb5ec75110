// NaiveAlgorithm.cpp -- the loop of NaiveAlgorithm::startSimulation (NaiveAlgorithm.cpp:15-260)
// over the C ABI: initial accelerations, then per step leapfrog part 1, accelerations, leapfrog
// part 2, with positions/velocities/|a|/energy captured on visualised steps.
#include "NaiveAlgorithm.hpp"

#include <chrono>
#include <cmath>
#include <iostream>

NaiveAlgorithm::NaiveAlgorithm(double dt, double tEnd, double vs, std::string& outDir)
    : nBodyAlgorithm(dt, tEnd, vs, outDir) {
    description = "Naive Algorithm";
}

void NaiveAlgorithm::computeAccelerations() {
    nb_throw_if(nb_naive_accel(ctx, d_m, d_x, d_y, d_z, d_ax, d_ay, d_az, n, G,
                               configuration::epsilon2, precisionMode(),
                               configuration::naive_algorithm::blockSize, nullptr),
                "nb_naive_accel");
    sync();
}

void NaiveAlgorithm::startSimulation(const SimulationData& d) {
    using clk = std::chrono::steady_clock;
    auto ms = [](clk::time_point a, clk::time_point b) {
        return std::chrono::duration<double, std::milli>(b - a).count();
    };
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
    auto a0 = clk::now();
    computeAccelerations();
    timer.addTimeToSequence("Acceleration Kernel Time", ms(a0, clk::now()));
    if (configuration::compute_energy) computeEnergy(step);
    storeAccelerations(step);
    std::cout << "Finished initial step " << step << std::endl << std::endl;
    time += dt;
    sinceVis += dt;
    step += 1;
    while (time <= t_end + 0.000001) {
        const bool vis = std::abs(sinceVis - visualizationStepWidth) < 0.000001;
        auto t0 = clk::now();
        leapfrogPart1();
        timer.addTimeToSequence("Leapfrog Part 1", ms(t0, clk::now()));
        if (vis) {
            download(d_x, positions_x[step]);
            download(d_y, positions_y[step]);
            download(d_z, positions_z[step]);
        }
        auto t1 = clk::now();
        computeAccelerations();
        timer.addTimeToSequence("Acceleration Kernel Time", ms(t1, clk::now()));
        auto t2 = clk::now();
        leapfrogPart2();
        timer.addTimeToSequence("Leapfrog Part 2", ms(t2, clk::now()));
        if (vis) {
            std::cout << "Finished step " << step << std::endl << std::endl;
            storeAccelerations(step);
            download(d_vx, velocities_x[step]);
            download(d_vy, velocities_y[step]);
            download(d_vz, velocities_z[step]);
            if (configuration::compute_energy) computeEnergy(step);
            step += 1;
            sinceVis = 0.0;
        }
        time += dt;
        sinceVis += dt;
    }
}
