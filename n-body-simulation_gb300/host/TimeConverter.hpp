// TimeConverter.hpp -- "<double><h|d|m|y>" to Earth days (src/utility/TimeConverter.hpp).
#pragma once
#include <string>

class TimeConverter {
public:
    // Throws std::invalid_argument unless the whole prefix is a number and the last character is
    // h (1/24 d), d, m (30.4167 d) or y (365.25 d) -- TimeConverter.cpp:4-48.
    static double convertToEarthDays(std::string& time);
};
