// BarnesHutAlgorithm.cpp -- the loop of BarnesHutAlgorithm::startSimulation
// (BarnesHutAlgorithm.cpp:18-278) over the C ABI, with the reference's timer keys. All work goes
// to one stream and the host waits only at visualised steps (see nBodyAlgorithm.hpp). With
// --graph, steps that are not visualised are replayed from a CUDA graph of one step.
//
// --opening=learned (no reference counterpart) runs the learned opening policy of a policy file
// (nb_policy_load) with FP32 pair arithmetic. The policy scales its decisions by each group's
// |a| of the previous evaluation, so the initial evaluation runs twice: the group theta rule
// (--theta) for a first |a|, then the policy.
#include "BarnesHutAlgorithm.hpp"

#include <cuda_runtime.h>

#include <cmath>
#include <iostream>
#include <stdexcept>

BarnesHutAlgorithm::BarnesHutAlgorithm(double dt, double tEnd, double vs, std::string& outDir)
    : nBodyAlgorithm(dt, tEnd, vs, outDir) {
    description = "Barnes-Hut Algorithm";
}

BarnesHutAlgorithm::~BarnesHutAlgorithm() {
    if (stepGraph) nb_graph_destroy(stepGraph);
    nb_bh_tree_destroy(octree);
    if (d_policy) cudaFree(d_policy);
}

nb_opening BarnesHutAlgorithm::openingRule() const {
    if (configuration::opening == "theta") return NB_OPEN_THETA;
    if (configuration::opening == "group") return NB_OPEN_THETA_GROUP;
    if (configuration::opening == "learned") return NB_OPEN_LEARNED;
    throw std::invalid_argument("opening must be theta, group or learned");
}

void BarnesHutAlgorithm::buildOctree() {
    nb_throw_if(nb_bh_build(ctx, octree, d_m, d_x, d_y, d_z, n, G, stream), "nb_bh_build");
}

void BarnesHutAlgorithm::computeAccelerations() {
    nb_throw_if(nb_bh_accel(ctx, octree, d_x, d_y, d_z, d_ax, d_ay, d_az, G,
                            configuration::epsilon2, openingRule(), precisionMode(), stream),
                "nb_bh_accel");
}

void BarnesHutAlgorithm::loadPolicy() {
    std::vector<float> params(NB_MLP_PARAMS);
    float log10_tau = 0.f;
    double theta_fallback = 0.0;
    uint32_t count_cap = 0, flags = 0;
    nb_throw_if(nb_policy_load(configuration::policyFile.c_str(), params.data(), &log10_tau,
                               &theta_fallback, &count_cap, &flags),
                "nb_policy_load");
    if (cudaMalloc(&d_policy, params.size() * sizeof(float)) != cudaSuccess ||
        cudaMemcpy(d_policy, params.data(), params.size() * sizeof(float),
                   cudaMemcpyHostToDevice) != cudaSuccess)
        throw std::runtime_error("cannot place the opening policy on the device");
    nb_throw_if(nb_bh_set_policy(octree, d_policy, log10_tau, theta_fallback, count_cap, flags),
                "nb_bh_set_policy");
}

void BarnesHutAlgorithm::startSimulation(const SimulationData& d) {
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
    // double-float terms for df64); for f32c none beyond the FP32 records, and quantized keys;
    // the learned policy's records for --opening=learned
    const nb_precision prec = precisionMode();
    const nb_opening rule = openingRule();
    unsigned int records = prec == NB_F32C ? NB_BUILD_QUANTIZED_KEYS : NB_REC_FP64;
    if (prec == NB_DF64) records |= NB_REC_DF;
    if (rule == NB_OPEN_LEARNED) {
        if (prec != NB_F32C)
            throw std::invalid_argument("--opening=learned runs FP32 pair arithmetic: "
                                        "use --precision=f32c");
        records = NB_REC_LEARNED | NB_BUILD_QUANTIZED_KEYS;
    }
    nb_throw_if(nb_bh_set_records(octree, records), "nb_bh_set_records");
    if (rule == NB_OPEN_LEARNED) loadPolicy();

    timer.setProperties(description, n, deviceName);
    for (const char* k : {"Total Time", "Octree creation", "Acceleration Kernel Time",
                          "Leapfrog Part 1", "Leapfrog Part 2"})
        timer.addTimingSequence(k);

    double time = 0.0, sinceVis = 0.0;
    d_type::int_t step = 0;
    const int b0 = phases.mark(stream);
    buildOctree();
    const int b1 = phases.mark(stream);
    if (rule == NB_OPEN_LEARNED)  // a first |a| for the policy's scale
        nb_throw_if(nb_bh_accel(ctx, octree, d_x, d_y, d_z, d_ax, d_ay, d_az, G,
                                configuration::epsilon2, NB_OPEN_THETA_GROUP, NB_F32C, stream),
                    "nb_bh_accel");
    computeAccelerations();
    const int b2 = phases.mark(stream);
    phases.span("Octree creation", b0, b1);
    phases.span("Acceleration Kernel Time", b1, b2);
    phases.span("Total Time", b0, b2);
    std::cout << std::endl;
    storeAccelerations(step);
    if (configuration::compute_energy) computeEnergy(step);
    finishVisualisedStep(step, d);
    std::cout << "Finished initial step " << step << std::endl << std::endl;
    if (configuration::useGraph) {
        timer.addTimingSequence("Leapfrog step (CUDA graph)");
        nb_throw_if(nb_bh_graph_create(ctx, octree, d_m, d_x, d_y, d_z, d_vx, d_vy, d_vz, d_vhx,
                                       d_vhy, d_vhz, d_ax, d_ay, d_az, n, G,
                                       configuration::epsilon2, dt, 1, rule, prec, &stepGraph),
                    "nb_bh_graph_create");
    }
    time += dt;
    sinceVis += dt;
    step += 1;
    while (time <= t_end + 0.000001) {
        const bool vis = std::abs(sinceVis - visualizationStepWidth) < 0.000001;
        if (!vis && stepGraph) {  // leapfrog part 1, build, traversal, part 2 in one launch
            const int g0 = phases.mark(stream);
            nb_throw_if(nb_graph_launch(stepGraph, stream), "nb_graph_launch");
            phases.span("Leapfrog step (CUDA graph)", g0, phases.mark(stream));
        } else {
            const int t0 = phases.mark(stream);
            leapfrogPart1();
            const int t1 = phases.mark(stream);
            if (vis) stagePositions();
            const int c0 = phases.mark(stream);
            buildOctree();
            const int c1 = phases.mark(stream);
            computeAccelerations();
            const int c2 = phases.mark(stream);
            leapfrogPart2();
            const int t2 = phases.mark(stream);
            phases.span("Leapfrog Part 1", t0, t1);
            phases.span("Octree creation", c0, c1);
            phases.span("Acceleration Kernel Time", c1, c2);
            phases.span("Total Time", c0, c2);
            phases.span("Leapfrog Part 2", c2, t2);
        }
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
