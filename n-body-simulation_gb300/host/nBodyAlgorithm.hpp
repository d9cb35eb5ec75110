// nBodyAlgorithm.hpp -- simulation shell over the C ABI: output capture, energy, ParaView
// output. Mirrors src/simulationBackend/nBodyAlgorithm.hpp:19-109 (same members and methods);
// the SYCL buffers become device arrays owned by the object and the kernels calls into
// libnbody_cuda.so.
//
// Unlike the reference, whose every kernel submission waits for the device (.wait()), the loop
// here enqueues all work on one CUDA stream and only waits at visualised steps and at the end:
// phase durations come from CUDA events read back at those points, visualised arrays are copied
// into pinned staging buffers on the stream, and the .vtp files of visualised steps are written
// by a background thread while the simulation goes on.
#pragma once

#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "Configuration.hpp"
#include "SimulationData.hpp"
#include "TimeMeasurement.hpp"
#include "nbody.h"

// Turns an nb_status into the reference's exception style.
void nb_throw_if(nb_status st, const char* what);

// Durations of named phases from CUDA events on a stream, resolved in batches: mark() records an
// event, span() pairs two marks under a timing-sequence name, flush() waits for the last mark and
// appends every pending span (ms) to a TimeMeasurement, returning the events to a pool.
class PhaseTimer {
public:
    ~PhaseTimer();
    int mark(nb_stream_t stream);
    void span(const std::string& sequence, int from, int to);
    void flush(TimeMeasurement& timer);
    size_t pending() const { return marks.size(); }

private:
    std::vector<void*> pool;   // cudaEvent_t
    std::vector<void*> marks;  // events recorded since the last flush
    std::vector<std::pair<std::string, std::pair<int, int>>> spans;
};

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
    nb_stream_t stream = nullptr;  // every launch and copy of the run
    d_type::int_t n = 0;
    double *d_m = nullptr, *d_x = nullptr, *d_y = nullptr, *d_z = nullptr;
    double *d_vx = nullptr, *d_vy = nullptr, *d_vz = nullptr;
    double *d_ax = nullptr, *d_ay = nullptr, *d_az = nullptr;
    double *d_vhx = nullptr, *d_vhy = nullptr, *d_vhz = nullptr;
    double* d_energy = nullptr;
    std::string deviceName;
    PhaseTimer phases;

    void upload(const SimulationData& simulationData);
    nb_precision precisionMode() const;
    void leapfrogPart1();
    void leapfrogPart2();
    // Waits for the stream, checks the device error word and moves the pending phase times into
    // `timer`; also done every few hundred marks so that the event pool stays bounded.
    void sync();
    void syncIfManyPending();

    // Visualised step `step`: positions are staged right after leapfrog part 1 (stagePositions),
    // velocities, |a| and energies after part 2 (stageVelocitiesAndAccelerations); finishStep
    // waits for the stream, moves the staged data into the output maps and hands the step to
    // the .vtp writer.
    void stagePositions();
    void stageVelocitiesAndAccelerations(d_type::int_t step);
    void finishVisualisedStep(d_type::int_t step, const SimulationData& d);

private:
    double* h_stage = nullptr;  // pinned: x, y, z, vx, vy, vz, ax, ay, az (n each), energy (4)
    bool energy_staged = false;

    // background .vtp writer
    struct VtpJob {
        size_t step;
        const std::vector<double>*px, *py, *pz, *vx, *vy, *vz, *acc;
        double energy[4];
    };
    std::thread writer;
    std::mutex writer_mutex;
    std::condition_variable writer_cv;
    std::deque<VtpJob> writer_jobs;
    bool writer_stop = false;
    std::string writer_error;
    const SimulationData* writer_data = nullptr;
    std::string runDirectory();
    void writerLoop();
    void stopWriter();
    void writeVtp(const VtpJob& job, const SimulationData& data, const std::string& path);
};
