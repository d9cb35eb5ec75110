// Configuration.hpp -- run configuration of the host driver. Mirrors the reference's
// `configuration` namespace (src/utility/Configuration.hpp:12-124): same names, defaults
// (Configuration.cpp:5-22) and size rules (initializeConfigValues, Configuration.cpp:24-33).
#pragma once

#include <cstdint>
#include <string>

namespace d_type {
typedef unsigned int int_t;  // Configuration.hpp:8-10
}

namespace configuration {
extern d_type::int_t numberOfBodies;
extern double epsilon2;
extern bool compute_energy;
extern bool use_GPUs;
// additions of this build (no reference counterpart): the reference fixes G in AU^3 kg^-1 d^-2
// and FP64 pair arithmetic; these select another unit system and the precision form
extern double G;             // 0 = the reference's G (nBodyAlgorithm.hpp:55-61)
extern std::string precision;  // "f64" (default), "f64_ieee", "f32c", "df64"
extern std::string opening;    // "theta" (default, the reference's rule), "group", "learned"
extern std::string policyFile; // opening-policy file of --opening=learned (nb_policy_load)
extern bool useGraph;          // replay unvisualised Barnes-Hut steps from a captured CUDA graph

namespace naive_algorithm {
extern int blockSize;
extern int optimization_stage;
}  // namespace naive_algorithm

namespace barnes_hut_algorithm {
extern double theta;
extern int workGroupSize;
extern d_type::int_t stackSize;
extern d_type::int_t storageSizeParameter;
extern int AABBWorkItemCount;
extern int octreeWorkItemCount;
extern int octreeTopWorkItemCount;
extern int centerOfMassWorkItemCount;
extern int maxBuildLevel;
extern bool sortBodies;
}  // namespace barnes_hut_algorithm

void initializeConfigValues(d_type::int_t bodyCount, int storageSizeParam, int stackSizeParam);
void setBlockSize(int blockSize);
void setTheta(double theta);
void setAABBWorkItemCount(int workItemCount);
void setOctreeWorkItemCount(int workItemCount);
void setOctreeTopWorkItemCount(int workItemCount);
void setCenterOfMassWorkItemCount(int workItemCount);
void setMaxBuildLevel(int maxLevel);
void setEnergyComputation(bool computeEnergy);
void setSortBodies(bool sort_bodies);
void setDeviceGPU(bool useGPU);
void setWorkGroupSizeBarnesHut(int workGroupSize);
void setOptimizationStage(int stage);
}  // namespace configuration
