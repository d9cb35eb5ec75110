// TimeConverter.cpp -- conversion of the CLI's time strings, with the reference's factors and
// error behaviour (TimeConverter.cpp:4-48).
#include "TimeConverter.hpp"

#include <stdexcept>

double TimeConverter::convertToEarthDays(std::string& time) {
    static const char* kFormat = "Time values have to be of the format <double><h|d|m|y>";
    if (time.empty()) throw std::invalid_argument(kFormat);
    const char unit = time.back();
    const std::string number = time.substr(0, time.size() - 1);
    double value = 0;
    size_t used = 0;
    try {
        value = std::stod(number, &used);
    } catch (const std::exception&) {
        throw std::invalid_argument(kFormat);
    }
    if (used != number.size()) throw std::invalid_argument(kFormat);
    switch (unit) {
        case 'h': return value * (1.0 / 24);
        case 'd': return value;
        case 'm': return value * 30.4167;
        case 'y': return value * 365.25;
        default: throw std::invalid_argument(kFormat);
    }
}
