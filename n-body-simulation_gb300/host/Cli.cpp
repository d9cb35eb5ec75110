// Cli.cpp -- see Cli.hpp.
#include "Cli.hpp"

#include <algorithm>
#include <stdexcept>

const std::vector<std::string>& Cli::known() {
    static const std::vector<std::string> k = {
        // the reference's options (src/main.cpp:13-97)
        "file", "dt", "t_end", "vs", "vs_dir", "theta", "num_wi_octree", "num_wi_top_octree",
        "num_wi_AABB", "num_wi_com", "max_level_top_octree", "storage_size_param",
        "stack_size_param", "block_size", "algorithm", "energy", "sort_bodies", "use_gpus",
        "wg_size_barnes_hut", "opt_stage",
        // additions: unit system, softening, arithmetic, opening rule and its policy file,
        // graph replay of Barnes-Hut steps
        "G", "epsilon2", "precision", "opening", "policy", "graph", "help"};
    return k;
}

static bool is_bool_option(const std::string& k) {
    return k == "energy" || k == "sort_bodies" || k == "use_gpus" || k == "graph" || k == "help";
}

Cli::Cli(int argc, char** argv) {
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        if (a.rfind("--", 0) != 0) throw std::invalid_argument("unexpected argument " + a);
        a = a.substr(2);
        std::string key = a, val;
        const size_t eq = a.find('=');
        if (eq != std::string::npos) {
            key = a.substr(0, eq);
            val = a.substr(eq + 1);
        } else if (is_bool_option(key) &&
                   (i + 1 >= argc || std::string(argv[i + 1]).rfind("--", 0) == 0)) {
            val = "true";
        } else {
            if (i + 1 >= argc) throw std::invalid_argument("option --" + key + " needs a value");
            val = argv[++i];
        }
        if (std::find(known().begin(), known().end(), key) == known().end())
            throw std::invalid_argument("unknown option --" + key);
        values[key] = val;
    }
}

std::string Cli::str(const std::string& key) const {
    auto it = values.find(key);
    if (it == values.end()) throw std::invalid_argument("missing option --" + key);
    return it->second;
}

int Cli::integer(const std::string& key) const {
    const std::string v = str(key);
    size_t used = 0;
    const int r = std::stoi(v, &used);
    if (used != v.size()) throw std::invalid_argument("--" + key + " expects an integer");
    return r;
}

double Cli::number(const std::string& key) const {
    const std::string v = str(key);
    size_t used = 0;
    const double r = std::stod(v, &used);
    if (used != v.size()) throw std::invalid_argument("--" + key + " expects a number");
    return r;
}

bool Cli::flag(const std::string& key) const {
    std::string v = str(key);
    std::transform(v.begin(), v.end(), v.begin(), ::tolower);
    if (v == "true" || v == "1" || v == "yes") return true;
    if (v == "false" || v == "0" || v == "no") return false;
    throw std::invalid_argument("--" + key + " expects true or false");
}
