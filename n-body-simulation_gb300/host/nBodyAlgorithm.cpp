// nBodyAlgorithm.cpp -- shared simulation shell (nBodyAlgorithm.cpp:11-411 of the reference:
// energy, |a| capture, velocity adjustment, ParaView .pvd/.vtp, lastState.csv, times.json).
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
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, 0) == cudaSuccess) deviceName = prop.name;
}

nBodyAlgorithm::~nBodyAlgorithm() {
    for (double* p : {d_m, d_x, d_y, d_z, d_vx, d_vy, d_vz, d_ax, d_ay, d_az, d_vhx, d_vhy, d_vhz,
                      d_energy})
        if (p) cudaFree(p);
    nb_ctx_destroy(ctx);
}

void nBodyAlgorithm::upload(const SimulationData& d) {
    n = (d_type::int_t)d.mass.size();
    const size_t bytes = (size_t)n * sizeof(double);
    double** arrs[] = {&d_m, &d_x, &d_y, &d_z, &d_vx, &d_vy, &d_vz, &d_ax,
                       &d_ay, &d_az, &d_vhx, &d_vhy, &d_vhz};
    for (double** a : arrs) cuda_throw_if(cudaMalloc(a, bytes), "cudaMalloc");
    cuda_throw_if(cudaMalloc(&d_energy, 4 * sizeof(double)), "cudaMalloc");
    const std::vector<double>* src[] = {&d.mass, &d.positions_x, &d.positions_y, &d.positions_z,
                                        &d.velocities_x, &d.velocities_y, &d.velocities_z};
    double* dst[] = {d_m, d_x, d_y, d_z, d_vx, d_vy, d_vz};
    for (int k = 0; k < 7; ++k)
        cuda_throw_if(cudaMemcpy(dst[k], src[k]->data(), bytes, cudaMemcpyHostToDevice), "upload");
    for (double* a : {d_ax, d_ay, d_az, d_vhx, d_vhy, d_vhz})
        cuda_throw_if(cudaMemset(a, 0, bytes), "cudaMemset");
}

void nBodyAlgorithm::download(const double* dev, std::vector<double>& host) const {
    host.resize(n);
    cuda_throw_if(cudaMemcpy(host.data(), dev, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost),
                  "download");
}

nb_precision nBodyAlgorithm::precisionMode() const {
    if (configuration::precision == "f64") return NB_F64;
    if (configuration::precision == "f64_ieee") return NB_F64_IEEE;
    if (configuration::precision == "f32c") return NB_F32C;
    if (configuration::precision == "df64") return NB_DF64;
    throw std::invalid_argument("precision must be f64, f64_ieee, f32c or df64");
}

void nBodyAlgorithm::sync() { nb_throw_if(nb_sync(ctx, nullptr), "nb_sync"); }

void nBodyAlgorithm::leapfrogPart1() {
    nb_throw_if(nb_leapfrog_kick_drift(ctx, d_vhx, d_vhy, d_vhz, d_vx, d_vy, d_vz, d_x, d_y, d_z,
                                       d_ax, d_ay, d_az, n, dt, nullptr),
                "leapfrog part 1");
    sync();
}

void nBodyAlgorithm::leapfrogPart2() {
    nb_throw_if(nb_leapfrog_kick(ctx, d_vx, d_vy, d_vz, d_vhx, d_vhy, d_vhz, d_ax, d_ay, d_az, n,
                                 dt, nullptr),
                "leapfrog part 2");
    sync();
}

// nBodyAlgorithm.cpp:11-86
void nBodyAlgorithm::computeEnergy(d_type::int_t step) {
    nb_throw_if(nb_energy(ctx, d_m, d_x, d_y, d_z, d_vx, d_vy, d_vz, n, G, d_energy, nullptr),
                "nb_energy");
    sync();
    double e[4];
    cuda_throw_if(cudaMemcpy(e, d_energy, sizeof(e), cudaMemcpyDeviceToHost), "energy");
    kineticEnergy[step] = e[0];
    potentialEnergy[step] = e[1];
    totalEnergy[step] = e[2];
    virialEquilibrium[step] = e[3];
}

// nBodyAlgorithm.cpp:88-102: keeps |a| only
void nBodyAlgorithm::storeAccelerations(d_type::int_t step) {
    std::vector<double> ax, ay, az;
    download(d_ax, ax);
    download(d_ay, ay);
    download(d_az, az);
    auto& out = acceleration[step];
    out.resize(n);
    for (d_type::int_t i = 0; i < n; ++i) out[i] = std::sqrt(ax[i] * ax[i] + ay[i] * ay[i] + az[i] * az[i]);
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

static int bodyClassCode(const std::string& c) {  // nBodyAlgorithm.cpp:298-342
    static const char* kClasses[] = {"AMO", "APO", "ATE", "IEO", "MCA", "IMB", "MBA", "OMB", "CEN",
                                     "TJN", "TNO", "AST", "PAA", "HYA", "STA", "DWA", "PLA", "SAT"};
    for (int k = 0; k < 18; ++k)
        if (c == kClasses[k]) return k + 1;
    return 0;
}

void nBodyAlgorithm::writeVtp(size_t i, const SimulationData& d, const std::string& path) {
    std::ofstream f(path);
    const size_t np = positions_x[i].size();
    f << "<?xml version=\"1.0\"?>" << '\n'
      << R"(<VTKFile type="PolyData" version="0.1" byte_order="LittleEndian" header_type="UInt64">)"
      << '\n'
      << "<PolyData>" << '\n'
      << "<Piece NumberOfPoints=\"" << np << "\" NumberOfVerts=\"" << np << "\">" << '\n'
      << "<Points>" << '\n'
      << R"(<DataArray type="Float64" Name="position" NumberOfComponents="3" format="ascii">)"
      << '\n';
    for (size_t j = 0; j < np; ++j)
        f << positions_x[i][j] << " " << positions_y[i][j] << " " << positions_z[i][j] << '\n';
    f << "</DataArray>" << '\n' << "</Points>" << '\n' << "<PointData>" << '\n'
      << R"(<DataArray type="Int32" Name="body_id" NumberOfComponents="1" format="ascii">)" << '\n';
    for (size_t j = 0; j < np; ++j) f << j << '\n';
    f << "</DataArray>" << '\n'
      << R"(<DataArray type="Float64" Name="velocity" NumberOfComponents="3" format="ascii">)"
      << '\n';
    for (size_t j = 0; j < velocities_x[i].size(); ++j)
        f << velocities_x[i][j] << " " << velocities_y[i][j] << " " << velocities_z[i][j] << '\n';
    f << "</DataArray>" << '\n'
      << R"(<DataArray type="Float64" Name="acceleration" NumberOfComponents="1" format="ascii">)"
      << '\n';
    for (size_t j = 0; j < np; ++j) f << acceleration[i][j] << '\n';
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
    std::map<d_type::int_t, double>* vals[] = {&kineticEnergy, &potentialEnergy, &totalEnergy,
                                              &virialEquilibrium};
    for (int k = 0; k < 4; ++k) {
        f << "<DataArray type=\"Float64\" Name=\"" << names[k]
          << "\" NumberOfTuples=\"1\" format=\"ascii\">" << '\n';
        if (e) f << (*vals[k])[(d_type::int_t)i] << '\n';
        else f << 0 << '\n';
        f << "</DataArray>" << '\n';
    }
    f << "</FieldData>" << '\n' << "</PolyData>" << '\n' << "</VTKFile>" << '\n';
}

// nBodyAlgorithm.cpp:129-251: <vs_dir>/<timestamp>/ with times.json, lastState.csv,
// simulation.pvd and simulation_step<i>.vtp
void nBodyAlgorithm::generateParaViewOutput(const SimulationData& d) {
    std::time_t now = std::time(nullptr);
    std::string stamp = std::ctime(&now);
    std::replace(stamp.begin(), stamp.end(), ' ', '_');
    stamp = stamp.substr(0, stamp.size() - 1);
    const std::string base = outputDirectory + '/' + stamp + '/';
    std::filesystem::create_directories(base);
    lastOutputPath = base;
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
        writeVtp(i, d, base + name);
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
