// main.cpp -- nbody_sim: the reference's command line (src/main.cpp:9-240) over the GB300
// library. Reads the CSV, configures the run, simulates with the naive or Barnes-Hut algorithm
// and writes ParaView output, lastState.csv and times.json.
#include <iostream>
#include <memory>
#include <stdexcept>

#include "BarnesHutAlgorithm.hpp"
#include "Cli.hpp"
#include "Configuration.hpp"
#include "InputParser.hpp"
#include "NaiveAlgorithm.hpp"
#include "TimeConverter.hpp"

static void usage() {
    std::cout << "usage: nbody_sim --file=<bodies.csv> --dt=<t> --t_end=<t> --vs=<t> --vs_dir=<dir>"
                 " --algorithm=<naive|BarnesHut> [options]\n"
                 "  times are <double><h|d|m|y>; options: --theta --block_size --opt_stage"
                 " --energy --sort_bodies --max_level_top_octree --storage_size_param"
                 " --stack_size_param --num_wi_* --wg_size_barnes_hut --use_gpus"
                 " --G --epsilon2 --precision=<f64|f64_ieee|f32c|df64>"
                 " --opening=<theta|group|learned> --policy=<file> --graph\n";
}

static int run(int argc, char** argv) {
    Cli options(argc, argv);
    if (options.has("help")) {
        usage();
        return 0;
    }
    std::string path = options.str("file");
    std::string outputDirectoryPath = options.str("vs_dir");
    std::string dt_input = options.str("dt"), t_end_input = options.str("t_end"),
                vs_input = options.str("vs");
    const double dt = TimeConverter::convertToEarthDays(dt_input);
    const double t_end = TimeConverter::convertToEarthDays(t_end_input);
    const double vs = TimeConverter::convertToEarthDays(vs_input);

    SimulationData simulationData;
    InputParser::parse_input(path, simulationData);
    if (simulationData.mass.empty()) throw std::invalid_argument("the input file holds no bodies");

    const int storage = options.has("storage_size_param") ? options.integer("storage_size_param") : 16;
    const int stack = options.has("stack_size_param") ? options.integer("stack_size_param") : 16;
    configuration::initializeConfigValues((d_type::int_t)simulationData.mass.size(), storage, stack);
    if (options.has("energy")) configuration::setEnergyComputation(options.flag("energy"));
    if (options.has("use_gpus")) configuration::setDeviceGPU(options.flag("use_gpus"));
    if (options.has("G")) configuration::G = options.number("G");
    if (options.has("epsilon2")) configuration::epsilon2 = options.number("epsilon2");
    if (options.has("precision")) configuration::precision = options.str("precision");
    if (options.has("opening")) configuration::opening = options.str("opening");
    if (options.has("policy")) configuration::policyFile = options.str("policy");
    if (options.has("graph")) configuration::useGraph = options.flag("graph");
    if (configuration::opening == "learned" && configuration::policyFile.empty())
        throw std::invalid_argument("--opening=learned needs --policy=<file>");

    const std::string algorithm = options.str("algorithm");
    if (algorithm == "naive") {
        if (options.has("block_size")) configuration::setBlockSize(options.integer("block_size"));
        if (options.has("opt_stage")) {
            const int s = options.integer("opt_stage");
            if (s > 2 || s < 0) throw std::invalid_argument("Optimization stage must be 0,1 or 2");
            configuration::setOptimizationStage(s);
        }
        std::cout << "Naive algorithm configuration:" << std::endl
                  << "Block Size ------------------------------------ "
                  << configuration::naive_algorithm::blockSize << std::endl
                  << "Optimization stage acceleration kernel -------- "
                  << configuration::naive_algorithm::optimization_stage << std::endl
                  << "Precision ------------------------------------- " << configuration::precision
                  << std::endl << std::endl;
    } else if (algorithm == "BarnesHut") {
        namespace bh = configuration::barnes_hut_algorithm;
        if (options.has("theta")) configuration::setTheta(options.number("theta"));
        if (options.has("num_wi_octree")) configuration::setOctreeWorkItemCount(options.integer("num_wi_octree"));
        if (options.has("num_wi_top_octree"))
            configuration::setOctreeTopWorkItemCount(options.integer("num_wi_top_octree"));
        if (options.has("num_wi_com")) configuration::setCenterOfMassWorkItemCount(options.integer("num_wi_com"));
        if (options.has("max_level_top_octree"))
            configuration::setMaxBuildLevel(options.integer("max_level_top_octree"));
        if (options.has("num_wi_AABB")) configuration::setAABBWorkItemCount(options.integer("num_wi_AABB"));
        if (options.has("sort_bodies")) configuration::setSortBodies(options.flag("sort_bodies"));
        if (options.has("wg_size_barnes_hut"))
            configuration::setWorkGroupSizeBarnesHut(options.integer("wg_size_barnes_hut"));
        std::cout << "Barnes-Hut algorithm configuration:" << std::endl
                  << "Theta ----------------------------------- " << bh::theta << std::endl
                  << "Maximum build level top of octree ------- " << bh::maxBuildLevel << std::endl
                  << "Sort Bodies enabled --------------------- " << bh::sortBodies << std::endl
                  << "Precision / opening rule ---------------- " << configuration::precision
                  << " / " << configuration::opening << std::endl << std::endl;
    } else {
        throw std::invalid_argument("Algorithm must either be <naive> or <BarnesHut>");
    }

    std::unique_ptr<nBodyAlgorithm> algo;
    if (algorithm == "naive") algo = std::make_unique<NaiveAlgorithm>(dt, t_end, vs, outputDirectoryPath);
    else algo = std::make_unique<BarnesHutAlgorithm>(dt, t_end, vs, outputDirectoryPath);
    algo->startSimulation(simulationData);
    algo->generateParaViewOutput(simulationData);
    std::cout << "Output written to " << algo->lastOutputPath << std::endl;
    return 0;
}

int main(int argc, char** argv) {
    try {
        return run(argc, argv);
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << std::endl;
        return 1;
    }
}
