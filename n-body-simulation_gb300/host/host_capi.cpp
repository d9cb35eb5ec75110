// host_capi.cpp -- C entry points of libnbody_host.so that expose the host-side logic (CSV
// splitting, time strings, option parsing) to tests without a GPU.
#include <cstring>
#include <stdexcept>
#include <string>

#include "Cli.hpp"
#include "InputParser.hpp"
#include "TimeConverter.hpp"

extern "C" {

// Number of fields of `line`; field k copied (NUL-terminated) into out when k < count.
int nbh_split_string(const char* line, int k, char* out, int cap) {
    auto t = InputParser::splitString(line ? line : "");
    if (out && k >= 0 && k < (int)t.size() && cap > 0) {
        std::strncpy(out, t[k].c_str(), (size_t)cap - 1);
        out[cap - 1] = '\0';
    }
    return (int)t.size();
}

// 0 on success, 1 when the reference would throw std::invalid_argument.
int nbh_convert_to_earth_days(const char* s, double* out) {
    try {
        std::string v = s ? s : "";
        *out = TimeConverter::convertToEarthDays(v);
        return 0;
    } catch (const std::invalid_argument&) {
        return 1;
    }
}

// Number of bodies read, or -1 if the file cannot be parsed.
long long nbh_parse_input_count(const char* path, double* first_row7) {
    try {
        std::string p = path;
        SimulationData d;
        InputParser::parse_input(p, d);
        if (first_row7 && !d.mass.empty()) {
            const double v[7] = {d.mass[0], d.positions_x[0], d.positions_y[0], d.positions_z[0],
                                 d.velocities_x[0], d.velocities_y[0], d.velocities_z[0]};
            std::memcpy(first_row7, v, sizeof(v));
        }
        return (long long)d.mass.size();
    } catch (const std::exception&) {
        return -1;
    }
}

// 0 if the options parse, 1 otherwise.
int nbh_parse_options(int argc, char** argv) {
    try {
        Cli c(argc, argv);
        return 0;
    } catch (const std::exception&) {
        return 1;
    }
}

}  // extern "C"
