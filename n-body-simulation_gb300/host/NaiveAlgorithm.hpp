// NaiveAlgorithm.hpp -- all-pairs simulation (src/simulationBackend/NaiveAlgorithm.hpp).
#pragma once
#include "nBodyAlgorithm.hpp"

class NaiveAlgorithm : public nBodyAlgorithm {
public:
    NaiveAlgorithm(double dt, double tEnd, double visualizationStepWidth,
                   std::string& outputDirectory);
    void startSimulation(const SimulationData& simulationData) override;
    // NaiveAlgorithm::computeAccelerations_opt_{0,1,2} -> nb_naive_accel (all stages compute the
    // same sum; opt_stage and block size are kept for the CLI and times.json)
    void computeAccelerations();
};
