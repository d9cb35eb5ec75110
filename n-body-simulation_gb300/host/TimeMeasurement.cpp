// TimeMeasurement.cpp -- times.json with the reference's keys and layout
// (TimeMeasurement.cpp:16-62): algorithm, device, the algorithm's configuration, body count,
// then every non-empty timing sequence in milliseconds.
#include "TimeMeasurement.hpp"

#include <fstream>

void TimeMeasurement::addTimingSequence(const std::string& name) { times[name] = {}; }

void TimeMeasurement::addTimeToSequence(const std::string& name, double t) {
    times[name].push_back(t);
}

void TimeMeasurement::setProperties(std::string& algorithm, d_type::int_t& count,
                                    std::string& dev) {
    algorithmType = algorithm;
    bodyCount = count;
    device = dev;
}

void TimeMeasurement::exportJSON(const std::string& path) {
    std::ofstream f(path);
    f << "{ \n";
    f << "  \"algorithm\": \"" << algorithmType << "\",\n";
    f << "  \"device\": \"" << device << "\",\n";
    if (algorithmType == "Naive Algorithm") {
        f << "  \"block size\": " << configuration::naive_algorithm::blockSize << ",\n";
        f << "  \"optimization stage\": " << configuration::naive_algorithm::optimization_stage
          << ",\n";
    } else {
        namespace bh = configuration::barnes_hut_algorithm;
        f << "  \"theta\": " << bh::theta << ",\n";
        f << "  \"work-group size acceleration\": " << bh::workGroupSize << ",\n";
        f << "  \"work-items AABB\": " << bh::AABBWorkItemCount << ",\n";
        f << "  \"work-items octree\": " << bh::octreeWorkItemCount << ",\n";
        f << "  \"work-items center of mass\": " << bh::centerOfMassWorkItemCount << ",\n";
        f << "  \"work-items top octree\": " << bh::octreeTopWorkItemCount << ",\n";
        f << "  \"max build-level top octree\": " << bh::maxBuildLevel << ",\n";
        f << "  \"bodies sorted\": " << bh::sortBodies << ",\n";
    }
    f << "  \"precision\": \"" << configuration::precision << "\",\n";
    f << "  \"body count\": " << bodyCount;
    for (auto& [name, seq] : times) {
        if (seq.empty()) continue;
        f << ",\n  \"" << name << "\": [";
        for (size_t i = 0; i + 1 < seq.size(); ++i) f << seq[i] << ", ";
        f << seq.back() << "]";
    }
    f << "\n}";
}
