// BarnesHutAlgorithm.hpp -- Barnes-Hut simulation (src/simulationBackend/BarnesHutAlgorithm.hpp).
#pragma once
#include "nBodyAlgorithm.hpp"

class BarnesHutAlgorithm : public nBodyAlgorithm {
public:
    nb_bh_tree* octree = nullptr;

    BarnesHutAlgorithm(double dt, double tEnd, double visualizationStepWidth,
                       std::string& outputDirectory);
    ~BarnesHutAlgorithm() override;
    void startSimulation(const SimulationData& simulationData) override;
    // octree.buildOctree -> nb_bh_build; computeAccelerations -> nb_bh_accel
    void buildOctree();
    void computeAccelerations();

private:
    nb_graph* stepGraph = nullptr;  // one captured leapfrog step (--graph)
    float* d_policy = nullptr;      // network of --opening=learned
    nb_opening openingRule() const;
    void loadPolicy();
};
