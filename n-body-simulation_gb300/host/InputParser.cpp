// InputParser.cpp -- CSV reader with the reference's column order (InputParser.cpp:7-51).
#include "InputParser.hpp"

#include <fstream>
#include <stdexcept>

std::vector<std::string> InputParser::splitString(std::string s) {
    std::vector<std::string> out;
    size_t start = 0;
    for (size_t i = 0; i < s.size(); ++i) {
        if (s[i] == ',') {
            out.push_back(s.substr(start, i - start));
            start = i + 1;
        }
    }
    out.push_back(s.substr(start));
    return out;
}

void InputParser::parse_input(std::string& path, SimulationData& d) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open input file " + path);
    std::string line;
    std::getline(in, line);  // header
    size_t row = 1;
    while (std::getline(in, line)) {
        ++row;
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (line.empty()) continue;
        auto t = splitString(line);
        if (t.size() < 10)
            throw std::runtime_error("input row " + std::to_string(row) + ": expected 10 columns");
        try {
            d.names.push_back(t[1]);
            d.body_classes.push_back(t[2]);
            d.mass.push_back(std::stod(t[3]));
            d.positions_x.push_back(std::stod(t[4]));
            d.positions_y.push_back(std::stod(t[5]));
            d.positions_z.push_back(std::stod(t[6]));
            d.velocities_x.push_back(std::stod(t[7]));
            d.velocities_y.push_back(std::stod(t[8]));
            d.velocities_z.push_back(std::stod(t[9]));
        } catch (const std::logic_error&) {
            throw std::runtime_error("input row " + std::to_string(row) + ": not a number");
        }
    }
}
