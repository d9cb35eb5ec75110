// Cli.hpp -- option parsing for the host driver: the reference's option names
// (src/main.cpp:13-97, parsed there by cxxopts) in --key=value, --key value and bare --flag forms.
#pragma once
#include <map>
#include <string>
#include <vector>

class Cli {
public:
    // Throws std::invalid_argument for unknown options or a missing value.
    Cli(int argc, char** argv);
    bool has(const std::string& key) const { return values.count(key) != 0; }
    std::string str(const std::string& key) const;   // throws if absent
    int integer(const std::string& key) const;
    double number(const std::string& key) const;
    bool flag(const std::string& key) const;
    static const std::vector<std::string>& known();

private:
    std::map<std::string, std::string> values;
};
