// Configuration.cpp -- defaults and size rules of the reference (Configuration.cpp:5-33).
#include "Configuration.hpp"

#include <cmath>

d_type::int_t configuration::numberOfBodies = 0;
double configuration::epsilon2 = 1e-22;
bool configuration::compute_energy = false;
bool configuration::use_GPUs = true;
double configuration::G = 0.0;
std::string configuration::precision = "f64";
std::string configuration::opening = "theta";
std::string configuration::policyFile;
bool configuration::useGraph = false;

int configuration::naive_algorithm::blockSize = 64;
int configuration::naive_algorithm::optimization_stage = 2;

d_type::int_t configuration::barnes_hut_algorithm::storageSizeParameter = 0;
int configuration::barnes_hut_algorithm::AABBWorkItemCount = 1024;
int configuration::barnes_hut_algorithm::octreeWorkItemCount = 640;
int configuration::barnes_hut_algorithm::octreeTopWorkItemCount = 1024;
int configuration::barnes_hut_algorithm::centerOfMassWorkItemCount = 1024;
double configuration::barnes_hut_algorithm::theta = 1.05;
int configuration::barnes_hut_algorithm::maxBuildLevel = 7;
d_type::int_t configuration::barnes_hut_algorithm::stackSize = 0;
bool configuration::barnes_hut_algorithm::sortBodies = true;
int configuration::barnes_hut_algorithm::workGroupSize = 64;

void configuration::initializeConfigValues(d_type::int_t bodyCount, int storageSizeParam,
                                           int stackSizeParam) {
    numberOfBodies = bodyCount;
    barnes_hut_algorithm::storageSizeParameter = storageSizeParam * numberOfBodies;
    const auto lg = (d_type::int_t)std::ceil(std::log2((double)bodyCount));
    barnes_hut_algorithm::stackSize =
        bodyCount < 15000 ? stackSizeParam * lg + 500 : stackSizeParam * lg;
}

void configuration::setBlockSize(int v) { naive_algorithm::blockSize = v; }
void configuration::setTheta(double v) { barnes_hut_algorithm::theta = v; }
void configuration::setAABBWorkItemCount(int v) { barnes_hut_algorithm::AABBWorkItemCount = v; }
void configuration::setOctreeWorkItemCount(int v) { barnes_hut_algorithm::octreeWorkItemCount = v; }
void configuration::setOctreeTopWorkItemCount(int v) {
    barnes_hut_algorithm::octreeTopWorkItemCount = v;
}
void configuration::setCenterOfMassWorkItemCount(int v) {
    barnes_hut_algorithm::centerOfMassWorkItemCount = v;
}
void configuration::setMaxBuildLevel(int v) { barnes_hut_algorithm::maxBuildLevel = v; }
void configuration::setEnergyComputation(bool v) { compute_energy = v; }
void configuration::setSortBodies(bool v) { barnes_hut_algorithm::sortBodies = v; }
void configuration::setDeviceGPU(bool v) { use_GPUs = v; }
void configuration::setWorkGroupSizeBarnesHut(int v) { barnes_hut_algorithm::workGroupSize = v; }
void configuration::setOptimizationStage(int v) { naive_algorithm::optimization_stage = v; }
