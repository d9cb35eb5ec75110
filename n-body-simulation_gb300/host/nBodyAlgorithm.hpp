// nBodyAlgorithm.hpp -- simulation shell over the C ABI: output capture, energy, ParaView
// output. Mirrors src/simulationBackend/nBodyAlgorithm.hpp:19-109 (same members and methods);
// the SYCL buffers become device arrays owned by the object and the kernels calls into
// libnbody_cuda.so.
#pragma once

#include <map>
#include <string>
#include <vector>

#include "Configuration.hpp"
#include "SimulationData.hpp"
#include "TimeMeasurement.hpp"
#include "nbody.h"

// Turns an nb_status into the reference's exception style.
void nb_throw_if(nb_status st, const char* what);

class nBodyAlgorithm {
public:
    std::string description;
    std::string outputDirectory;
    double dt, t_end, visualizationStepWidth, G;
    TimeMeasurement timer;
    std::map<d_type::int_t, std::vector<double>> positions_x, positions_y, positions_z;
    std::map<d_type::int_t, std::vector<double>> velocities_x, velocities_y, velocities_z;
    std::map<d_type::int_t, std::vector<double>> acceleration;
    std::map<d_type::int_t, double> kineticEnergy, potentialEnergy, totalEnergy, virialEquilibrium;
    std::string lastOutputPath;  // directory written by generateParaViewOutput

    nBodyAlgorithm(double dt, double t_end, double visualizationStepWidth,
                   std::string& outputDirectory);
    virtual ~nBodyAlgorithm();

    virtual void startSimulation(const SimulationData& simulationData) = 0;
    void generateParaViewOutput(const SimulationData& simulationData);
    void outputLastState(const std::string& path);
    void computeEnergy(d_type::int_t currentStep);
    void storeAccelerations(d_type::int_t currentStep);
    void adjustVelocities(const SimulationData& simulationData);

protected:
    // device state (FP64 structure of arrays)
    nb_ctx* ctx = nullptr;
    d_type::int_t n = 0;
    double *d_m = nullptr, *d_x = nullptr, *d_y = nullptr, *d_z = nullptr;
    double *d_vx = nullptr, *d_vy = nullptr, *d_vz = nullptr;
    double *d_ax = nullptr, *d_ay = nullptr, *d_az = nullptr;
    double *d_vhx = nullptr, *d_vhy = nullptr, *d_vhz = nullptr;
    double* d_energy = nullptr;
    std::string deviceName;

    void upload(const SimulationData& simulationData);
    void download(const double* dev, std::vector<double>& host) const;
    nb_precision precisionMode() const;
    void leapfrogPart1();
    void leapfrogPart2();
    void sync();

private:
    void writeVtp(size_t step, const SimulationData& data, const std::string& path);
};
