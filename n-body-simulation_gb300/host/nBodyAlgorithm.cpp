// nBodyAlgorithm.cpp -- shared simulation shell (nBodyAlgorithm.cpp:11-411 of the reference:
// energy, |a| capture, velocity adjustment, ParaView .pvd/.vtp, lastState.csv, times.json), with
// the stream, event timing, staging and background .vtp writing described in the header.
#include "nBodyAlgorithm.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <ctime>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <stdexcept>

void nb_throw_if(nb_status st, const char* what) {
    if (st != NB_OK)
        throw std::runtime_error(std::string(what) + ": " + nb_last_error_string());
}

static void cuda_throw_if(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// ---------------------------------------------------------------------------------------------
// PhaseTimer
// ---------------------------------------------------------------------------------------------
PhaseTimer::~PhaseTimer() {
    for (void* e : pool) cudaEventDestroy((cudaEvent_t)e);
    for (void* e : marks) cudaEventDestroy((cudaEvent_t)e);
}

int PhaseTimer::mark(nb_stream_t stream) {
    cudaEvent_t e = nullptr;
    if (!pool.empty()) {
        e = (cudaEvent_t)pool.back();
        pool.pop_back();
    } else {
        cuda_throw_if(cudaEventCreate(&e), "cudaEventCreate");
    }
    marks.push_back(e);
    cuda_throw_if(cudaEventRecord(e, (cudaStream_t)stream), "cudaEventRecord");
    return (int)marks.size() - 1;
}

void PhaseTimer::span(const std::string& sequence, int from, int to) {
    spans.push_back({sequence, {from, to}});
}

void PhaseTimer::flush(TimeMeasurement& timer) {
    if (marks.empty()) return;
    cuda_throw_if(cudaEventSynchronize((cudaEvent_t)marks.back()), "cudaEventSynchronize");
    for (auto& [name, ft] : spans) {
        float ms = 0.f;
        cuda_throw_if(cudaEventElapsedTime(&ms, (cudaEvent_t)marks[ft.first],
                                           (cudaEvent_t)marks[ft.second]),
                      "cudaEventElapsedTime");
        timer.addTimeToSequence(name, ms);
    }
    spans.clear();
    pool.insert(pool.end(), marks.begin(), marks.end());
    marks.clear();
}

// ---------------------------------------------------------------------------------------------
// nBodyAlgorithm
// ---------------------------------------------------------------------------------------------
nBodyAlgorithm::nBodyAlgorithm(double dt_, double t_end_, double vs, std::string& outDir)
    : outputDirectory(outDir), dt(dt_), t_end(t_end_), visualizationStepWidth(vs) {
    if (configuration::G != 0) {
        G = configuration::G;
    } else {  // nBodyAlgorithm.hpp:55-61
        G = 6.67428 * std::pow(10, -11);
        const double meter_AU = 1.0 / (1.49597870691 * std::pow(10, 11));
        const double second_days = 1.0 / 86400;
        G = G * (std::pow(meter_AU, 3) / std::pow(second_days, 2));
    }
    if (!configuration::use_GPUs)
        throw std::invalid_argument(
            "use_gpus=false: this build runs the force paths on the GPU only");
    nb_throw_if(nb_ctx_create(0, &ctx), "nb_ctx_create");
    cudaStream_t s = nullptr;
    cuda_throw_if(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
    stream = (nb_stream_t)s;
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, 0) == cudaSuccess) deviceName = prop.name;
}

nBodyAlgorithm::~nBodyAlgorithm() {
    try {
        stopWriter();
    } catch (...) {
    }
    if (stream) cudaStreamSynchronize((cudaStream_t)stream);
    for (double* p : {d_m, d_x, d_y, d_z, d_vx, d_vy, d_vz, d_ax, d_ay, d_az, d_vhx, d_vhy, d_vhz,
                      d_energy})
        if (p) cudaFree(p);
    if (h_stage) cudaFreeHost(h_stage);
    if (stream) cudaStreamDestroy((cudaStream_t)stream);
    nb_ctx_destroy(ctx);
}

void nBodyAlgorithm::upload(const SimulationData& d) {
    n = (d_type::int_t)d.mass.size();
    const size_t bytes = (size_t)n * sizeof(double);
    double** arrs[] = {&d_m, &d_x, &d_y, &d_z, &d_vx, &d_vy, &d_vz, &d_ax,
                       &d_ay, &d_az, &d_vhx, &d_vhy, &d_vhz};
    for (double** a : arrs) cuda_throw_if(cudaMalloc(a, bytes), "cudaMalloc");
    cuda_throw_if(cudaMalloc(&d_energy, 4 * sizeof(double)), "cudaMalloc");
    cuda_throw_if(cudaMallocHost(&h_stage, (9 * (size_t)n + 4) * sizeof(double)),
                  "cudaMallocHost");
    const std::vector<double>* src[] = {&d.mass, &d.positions_x, &d.positions_y, &d.positions_z,
                                        &d.velocities_x, &d.velocities_y, &d.velocities_z};
    double* dst[] = {d_m, d_x, d_y, d_z, d_vx, d_vy, d_vz};
    cudaStream_t s = (cudaStream_t)stream;
    for (int k = 0; k < 7; ++k)
        cuda_throw_if(cudaMemcpyAsync(dst[k], src[k]->data(), bytes, cudaMemcpyHostToDevice, s),
                      "upload");
    for (double* a : {d_ax, d_ay, d_az, d_vhx, d_vhy, d_vhz})
        cuda_throw_if(cudaMemsetAsync(a, 0, bytes, s), "cudaMemset");
    // the host vectors may change after this call returns
    cuda_throw_if(cudaStreamSynchronize(s), "upload");
}

nb_precision nBodyAlgorithm::precisionMode() const {
    if (configuration::precision == "f64") return NB_F64;
    if (configuration::precision == "f64_ieee") return NB_F64_IEEE;
    if (configuration::precision == "f32c") return NB_F32C;
    if (configuration::precision == "df64") return NB_DF64;
    throw std::invalid_argument("precision must be f64, f64_ieee, f32c or df64");
}

void nBodyAlgorithm::sync() {
    nb_throw_if(nb_sync(ctx, stream), "nb_sync");
    phases.flush(timer);
}

void nBodyAlgorithm::syncIfManyPending() {
    if (phases.pending() > 1024) sync();
}

void nBodyAlgorithm::leapfrogPart1() {
    nb_throw_if(nb_leapfrog_kick_drift(ctx, d_vhx, d_vhy, d_vhz, d_vx, d_vy, d_vz, d_x, d_y, d_z,
                                       d_ax, d_ay, d_az, n, dt, stream),
                "leapfrog part 1");
}

void nBodyAlgorithm::leapfrogPart2() {
    nb_throw_if(nb_leapfrog_kick(ctx, d_vx, d_vy, d_vz, d_vhx, d_vhy, d_vhz, d_ax, d_ay, d_az, n,
                                 dt, stream),
                "leapfrog part 2");
}

static void stage(double* host, const double* dev, size_t count, nb_stream_t s) {
    cuda_throw_if(cudaMemcpyAsync(host, dev, count * sizeof(double), cudaMemcpyDeviceToHost,
                                  (cudaStream_t)s),
                  "staging copy");
}

// nBodyAlgorithm.cpp:11-86 (the sums run on the GPU; the result is staged for the step)
void nBodyAlgorithm::computeEnergy(d_type::int_t) {
    nb_throw_if(nb_energy(ctx, d_m, d_x, d_y, d_z, d_vx, d_vy, d_vz, n, G, d_energy, stream),
                "nb_energy");
    stage(h_stage + 9 * (size_t)n, d_energy, 4, stream);
    energy_staged = true;
}

// nBodyAlgorithm.cpp:88-102 (|a| is formed when the step is finished)
void nBodyAlgorithm::storeAccelerations(d_type::int_t) {
    stage(h_stage + 6 * (size_t)n, d_ax, n, stream);
    stage(h_stage + 7 * (size_t)n, d_ay, n, stream);
    stage(h_stage + 8 * (size_t)n, d_az, n, stream);
}

void nBodyAlgorithm::stagePositions() {
    stage(h_stage + 0 * (size_t)n, d_x, n, stream);
    stage(h_stage + 1 * (size_t)n, d_y, n, stream);
    stage(h_stage + 2 * (size_t)n, d_z, n, stream);
}

void nBodyAlgorithm::stageVelocitiesAndAccelerations(d_type::int_t step) {
    stage(h_stage + 3 * (size_t)n, d_vx, n, stream);
    stage(h_stage + 4 * (size_t)n, d_vy, n, stream);
    stage(h_stage + 5 * (size_t)n, d_vz, n, stream);
    storeAccelerations(step);
    if (configuration::compute_energy) computeEnergy(step);
}

void nBodyAlgorithm::finishVisualisedStep(d_type::int_t step, const SimulationData& d) {
    sync();
    const size_t nn = n;
    const double* h = h_stage;
    if (step > 0) {  // step 0 keeps the input positions and the adjusted input velocities
        positions_x[step].assign(h, h + nn);
        positions_y[step].assign(h + nn, h + 2 * nn);
        positions_z[step].assign(h + 2 * nn, h + 3 * nn);
        velocities_x[step].assign(h + 3 * nn, h + 4 * nn);
        velocities_y[step].assign(h + 4 * nn, h + 5 * nn);
        velocities_z[step].assign(h + 5 * nn, h + 6 * nn);
    }
    auto& acc = acceleration[step];
    acc.resize(nn);
    const double *ax = h + 6 * nn, *ay = h + 7 * nn, *az = h + 8 * nn;
    for (size_t i = 0; i < nn; ++i) acc[i] = std::sqrt(ax[i] * ax[i] + ay[i] * ay[i] + az[i] * az[i]);
    VtpJob job{step, &positions_x[step], &positions_y[step], &positions_z[step],
               &velocities_x[step], &velocities_y[step], &velocities_z[step], &acc,
               {0, 0, 0, 0}};
    if (energy_staged) {
        const double* e = h + 9 * nn;
        kineticEnergy[step] = e[0];
        potentialEnergy[step] = e[1];
        totalEnergy[step] = e[2];
        virialEquilibrium[step] = e[3];
        for (int k = 0; k < 4; ++k) job.energy[k] = e[k];
        energy_staged = false;
    }
    {
        std::lock_guard<std::mutex> lock(writer_mutex);
        if (!writer_error.empty()) throw std::runtime_error("vtp writer: " + writer_error);
        writer_data = &d;
        writer_jobs.push_back(job);
        if (!writer.joinable()) {
            runDirectory();
            writer = std::thread(&nBodyAlgorithm::writerLoop, this);
        }
    }
    writer_cv.notify_one();
}

// nBodyAlgorithm.cpp:104-127: only the step-0 output velocities change
void nBodyAlgorithm::adjustVelocities(const SimulationData& d) {
    double sm = 0, sx = 0, sy = 0, sz = 0;
    for (size_t i = 0; i < d.mass.size(); ++i) {
        sm += d.mass[i];
        sx += d.mass[i] * d.velocities_x[i];
        sy += d.mass[i] * d.velocities_y[i];
        sz += d.mass[i] * d.velocities_z[i];
    }
    const double ux = sx / sm, uy = sy / sm, uz = sz / sm;
    for (size_t i = 0; i < d.mass.size(); ++i) {
        velocities_x[0][i] -= ux;
        velocities_y[0][i] -= uy;
        velocities_z[0][i] -= uz;
    }
}

// <vs_dir>/<timestamp>/, created when the first visualised step is handed to the writer
// (nBodyAlgorithm.cpp:129-251 names it by the time of the output)
std::string nBodyAlgorithm::runDirectory() {
    if (lastOutputPath.empty()) {
        std::time_t now = std::time(nullptr);
        std::string stamp = std::ctime(&now);
        std::replace(stamp.begin(), stamp.end(), ' ', '_');
        stamp = stamp.substr(0, stamp.size() - 1);
        lastOutputPath = outputDirectory + '/' + stamp + '/';
        std::filesystem::create_directories(lastOutputPath);
    }
    return lastOutputPath;
}

void nBodyAlgorithm::writerLoop() {
    for (;;) {
        VtpJob job{};
        const SimulationData* data = nullptr;
        std::string base;
        {
            std::unique_lock<std::mutex> lock(writer_mutex);
            writer_cv.wait(lock, [&] { return writer_stop || !writer_jobs.empty(); });
            if (writer_jobs.empty()) return;  // stop requested and nothing left
            job = writer_jobs.front();
            writer_jobs.pop_front();
            data = writer_data;
            base = lastOutputPath;
        }
        try {
            writeVtp(job, *data, base + "simulation_step" + std::to_string(job.step) + ".vtp");
        } catch (const std::exception& e) {
            std::lock_guard<std::mutex> lock(writer_mutex);
            writer_error = e.what();
            return;
        }
    }
}

void nBodyAlgorithm::stopWriter() {
    {
        std::lock_guard<std::mutex> lock(writer_mutex);
        writer_stop = true;
    }
    writer_cv.notify_all();
    if (writer.joinable()) writer.join();
    writer_stop = false;
    if (!writer_error.empty()) throw std::runtime_error("vtp writer: " + writer_error);
}

static int bodyClassCode(const std::string& c) {  // nBodyAlgorithm.cpp:298-342
    static const char* kClasses[] = {"AMO", "APO", "ATE", "IEO", "MCA", "IMB", "MBA", "OMB", "CEN",
                                     "TJN", "TNO", "AST", "PAA", "HYA", "STA", "DWA", "PLA", "SAT"};
    for (int k = 0; k < 18; ++k)
        if (c == kClasses[k]) return k + 1;
    return 0;
}

void nBodyAlgorithm::writeVtp(const VtpJob& job, const SimulationData& d, const std::string& path) {
    std::ofstream f(path);
    if (!f) throw std::runtime_error("cannot write " + path);
    const size_t np = job.px->size();
    f << "<?xml version=\"1.0\"?>" << '\n'
      << R"(<VTKFile type="PolyData" version="0.1" byte_order="LittleEndian" header_type="UInt64">)"
      << '\n'
      << "<PolyData>" << '\n'
      << "<Piece NumberOfPoints=\"" << np << "\" NumberOfVerts=\"" << np << "\">" << '\n'
      << "<Points>" << '\n'
      << R"(<DataArray type="Float64" Name="position" NumberOfComponents="3" format="ascii">)"
      << '\n';
    for (size_t j = 0; j < np; ++j)
        f << (*job.px)[j] << " " << (*job.py)[j] << " " << (*job.pz)[j] << '\n';
    f << "</DataArray>" << '\n' << "</Points>" << '\n' << "<PointData>" << '\n'
      << R"(<DataArray type="Int32" Name="body_id" NumberOfComponents="1" format="ascii">)" << '\n';
    for (size_t j = 0; j < np; ++j) f << j << '\n';
    f << "</DataArray>" << '\n'
      << R"(<DataArray type="Float64" Name="velocity" NumberOfComponents="3" format="ascii">)"
      << '\n';
    for (size_t j = 0; j < job.vx->size(); ++j)
        f << (*job.vx)[j] << " " << (*job.vy)[j] << " " << (*job.vz)[j] << '\n';
    f << "</DataArray>" << '\n'
      << R"(<DataArray type="Float64" Name="acceleration" NumberOfComponents="1" format="ascii">)"
      << '\n';
    for (size_t j = 0; j < np; ++j) f << (*job.acc)[j] << '\n';
    f << "</DataArray>" << '\n'
      << R"(<DataArray type="Float64" Name="mass" NumberOfComponents="1" format="ascii">)" << '\n';
    for (double m : d.mass) f << m << '\n';
    f << "</DataArray>" << '\n'
      << R"(<DataArray type="String" Name="name" NumberOfComponents="1" format="ascii">)" << '\n';
    for (const std::string& name : d.names) {
        for (char c : name) f << (int)c << ' ';
        f << " 0" << '\n';
    }
    f << "</DataArray>" << '\n'
      << R"(<DataArray type="Int32" Name="orbit_class" NumberOfComponents="1" format="ascii">)"
      << '\n';
    for (const std::string& c : d.body_classes) f << bodyClassCode(c) << '\n';
    f << "</DataArray>" << '\n' << "</PointData>" << '\n' << "<Verts>" << '\n'
      << R"(<DataArray type="Int64" Name="offsets">)" << '\n';
    for (size_t j = 1; j <= np; ++j) f << j << ' ';
    f << '\n' << "</DataArray>" << '\n' << R"(<DataArray type="Int64" Name="connectivity">)" << '\n';
    for (size_t j = 0; j < np; ++j) f << j << ' ';
    f << '\n' << "</DataArray>" << '\n' << "</Verts>" << '\n' << "</Piece>" << '\n'
      << "<FieldData>" << '\n';
    const bool e = configuration::compute_energy;
    const char* names[] = {"kinetic energy", "potential energy", "total energy",
                           "virial equilibrium"};
    for (int k = 0; k < 4; ++k) {
        f << "<DataArray type=\"Float64\" Name=\"" << names[k]
          << "\" NumberOfTuples=\"1\" format=\"ascii\">" << '\n';
        if (e) f << job.energy[k] << '\n';
        else f << 0 << '\n';
        f << "</DataArray>" << '\n';
    }
    f << "</FieldData>" << '\n' << "</PolyData>" << '\n' << "</VTKFile>" << '\n';
}

// nBodyAlgorithm.cpp:129-251: <vs_dir>/<timestamp>/ with times.json, lastState.csv,
// simulation.pvd and simulation_step<i>.vtp (the .vtp files were written by the background
// writer while the simulation ran; this waits for it)
void nBodyAlgorithm::generateParaViewOutput(const SimulationData& d) {
    stopWriter();
    const std::string base = runDirectory();
    timer.exportJSON(base + "times.json");
    outputLastState(base + "lastState.csv");
    std::ofstream pvd(base + "/simulation.pvd");
    pvd << "<?xml version=\"1.0\"?>" << '\n'
        << R"(<VTKFile type="Collection" version="0.1" byte_order="LittleEndian" compressor="vtkZLibDataCompressor">)"
        << '\n'
        << "<Collection>" << '\n';
    for (size_t i = 0; i < positions_x.size(); ++i) {
        const std::string name = "simulation_step" + std::to_string(i) + ".vtp";
        pvd << "<DataSet timestep=\"" << i << "\" " << R"(group="" part="0" file=")" << name
            << "\"/>" << '\n';
    }
    pvd << "</Collection>" << '\n' << "</VTKFile>" << '\n';
}

// nBodyAlgorithm.cpp:397-411
void nBodyAlgorithm::outputLastState(const std::string& path) {
    std::ofstream f(path);
    const d_type::int_t i = (d_type::int_t)positions_x.size() - 1;
    f << "position_x, position_y, position_z \n";
    for (size_t j = 0; j < positions_x[i].size(); ++j)
        f << positions_x[i][j] << "," << positions_y[i][j] << "," << positions_z[i][j] << '\n';
}
