// BarnesHutAlgorithm.cpp -- the loop of BarnesHutAlgorithm::startSimulation
// (BarnesHutAlgorithm.cpp:18-278) over the C ABI, with the reference's timer keys.
#include "BarnesHutAlgorithm.hpp"

#include <chrono>
#include <cmath>
#include <iostream>
#include <stdexcept>

BarnesHutAlgorithm::BarnesHutAlgorithm(double dt, double tEnd, double vs, std::string& outDir)
    : nBodyAlgorithm(dt, tEnd, vs, outDir) {
    description = "Barnes-Hut Algorithm";
}

BarnesHutAlgorithm::~BarnesHutAlgorithm() { nb_bh_tree_destroy(octree); }

void BarnesHutAlgorithm::buildOctree() {
    nb_throw_if(nb_bh_build(ctx, octree, d_m, d_x, d_y, d_z, n, G, nullptr), "nb_bh_build");
    sync();
}

void BarnesHutAlgorithm::computeAccelerations() {
    nb_opening op;
    if (configuration::opening == "theta") op = NB_OPEN_THETA;
    else if (configuration::opening == "group") op = NB_OPEN_THETA_GROUP;
    else throw std::invalid_argument("opening must be theta or group");
    nb_throw_if(nb_bh_accel(ctx, octree, d_x, d_y, d_z, d_ax, d_ay, d_az, G,
                            configuration::epsilon2, op, precisionMode(), nullptr),
                "nb_bh_accel");
    sync();
}

void BarnesHutAlgorithm::startSimulation(const SimulationData& d) {
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
    nb_bh_params p;
    nb_bh_params_default(&p);
    p.theta = configuration::barnes_hut_algorithm::theta;
    p.max_build_level = configuration::barnes_hut_algorithm::maxBuildLevel;
    p.sort_bodies = configuration::barnes_hut_algorithm::sortBodies ? 1 : 0;
    nb_throw_if(nb_bh_tree_create(ctx, n, &p, &octree), "nb_bh_tree_create");
    // only the node records this run's traversal reads: FP64 centres for the FP64 rules (and the
    // double-float terms for df64); for f32c none beyond the FP32 records, and quantized keys
    const nb_precision prec = precisionMode();
    unsigned int records = prec == NB_F32C ? NB_BUILD_QUANTIZED_KEYS : NB_REC_FP64;
    if (prec == NB_DF64) records |= NB_REC_DF;
    nb_throw_if(nb_bh_set_records(octree, records), "nb_bh_set_records");

    timer.setProperties(description, n, deviceName);
    for (const char* k : {"Total Time", "Octree creation", "Acceleration Kernel Time",
                          "Leapfrog Part 1", "Leapfrog Part 2"})
        timer.addTimingSequence(k);

    double time = 0.0, sinceVis = 0.0;
    d_type::int_t step = 0;
    auto b0 = clk::now();
    buildOctree();
    auto b1 = clk::now();
    computeAccelerations();
    auto b2 = clk::now();
    timer.addTimeToSequence("Octree creation", ms(b0, b1));
    timer.addTimeToSequence("Acceleration Kernel Time", ms(b1, b2));
    timer.addTimeToSequence("Total Time", ms(b0, b2));
    std::cout << std::endl;
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
        auto c0 = clk::now();
        buildOctree();
        auto c1 = clk::now();
        computeAccelerations();
        auto c2 = clk::now();
        timer.addTimeToSequence("Octree creation", ms(c0, c1));
        timer.addTimeToSequence("Acceleration Kernel Time", ms(c1, c2));
        timer.addTimeToSequence("Total Time", ms(c0, c2));
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
