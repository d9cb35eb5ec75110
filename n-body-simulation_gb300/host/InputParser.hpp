// InputParser.hpp -- the reference's CSV input (src/simulationData/InputParser.hpp).
#pragma once
#include <string>
#include <vector>

#include "SimulationData.hpp"

class InputParser {
public:
    // Layout id,name,class,mass,pos_x,pos_y,pos_z,vel_x,vel_y,vel_z; the first line is skipped
    // (InputParser.cpp:7-32). Throws std::runtime_error if the file cannot be read or a row is
    // short or not numeric.
    static void parse_input(std::string& path, SimulationData& simulationData);
    // Splits on ',' keeping empty fields (InputParser.cpp:34-51).
    static std::vector<std::string> splitString(std::string string);
};
