// nb_policy.cu -- opening-policy files: a trained network of the learned opening rule with the
// settings it was tuned for, so that a policy trained once (nbody/learned.py) can be used by the
// host driver (nbody_sim --opening=learned --policy=<file>) or any other caller of the C ABI.
//
// Text format (one item per line, numbers in C locale, floats with 9 significant digits so that
// FP32 values round-trip exactly):
//   nbody-gb300 opening policy 1
//   network 8 32 32 1 relu
//   log10_tau <float>
//   theta_fallback <double>
//   count_cap <uint32>
//   flags <uint32>
//   params 1377
//   <1377 lines: W1[8][32], b1[32], W2[32][32], b2[32], w3[32], b3>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "nb_internal.cuh"

namespace {

constexpr const char* kMagic = "nbody-gb300 opening policy 1";
constexpr const char* kNetwork = "network 8 32 32 1 relu";

bool read_line(FILE* f, std::string& line) {
    line.clear();
    int c;
    while ((c = std::fgetc(f)) != EOF && c != '\n') line.push_back((char)c);
    if (!line.empty() && line.back() == '\r') line.pop_back();
    return c != EOF || !line.empty();
}

// "<key> <value>" -> value text, or nullptr when the key does not match.
const char* value_of(const std::string& line, const char* key) {
    const size_t k = std::strlen(key);
    if (line.size() <= k + 1 || line.compare(0, k, key) != 0 || line[k] != ' ') return nullptr;
    return line.c_str() + k + 1;
}

bool parse_double(const char* s, double* out) {
    if (!s) return false;
    char* end = nullptr;
    errno = 0;
    const double v = std::strtod(s, &end);
    if (end == s || *end != '\0' || errno == ERANGE || !std::isfinite(v)) return false;
    *out = v;
    return true;
}

bool parse_u32(const char* s, uint32_t* out) {
    if (!s || *s == '-') return false;
    char* end = nullptr;
    errno = 0;
    const unsigned long long v = std::strtoull(s, &end, 10);
    if (end == s || *end != '\0' || errno == ERANGE || v > 0xffffffffull) return false;
    *out = (uint32_t)v;
    return true;
}

}  // namespace

extern "C" {

nb_status nb_policy_save(const char* path, const float* params_host, float log10_tau,
                         double theta_fallback, uint32_t count_cap, uint32_t flags) {
    if (!path || !params_host)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_policy_save: null argument");
    for (int i = 0; i < NB_MLP_PARAMS; ++i)
        if (!std::isfinite(params_host[i]))
            return nb::set_error(NB_ERR_INVALID_ARG, "nb_policy_save: parameter %d not finite", i);
    FILE* f = std::fopen(path, "w");
    if (!f) return nb::set_error(NB_ERR_INVALID_ARG, "nb_policy_save: cannot open %s", path);
    std::fprintf(f, "%s\n%s\nlog10_tau %.9g\ntheta_fallback %.17g\ncount_cap %u\nflags %u\n"
                    "params %d\n",
                 kMagic, kNetwork, (double)log10_tau, theta_fallback, count_cap, flags,
                 NB_MLP_PARAMS);
    for (int i = 0; i < NB_MLP_PARAMS; ++i) std::fprintf(f, "%.9g\n", (double)params_host[i]);
    const bool ok = std::ferror(f) == 0;
    if (std::fclose(f) != 0 || !ok)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_policy_save: write to %s failed", path);
    return NB_OK;
}

nb_status nb_policy_load(const char* path, float* params_host, float* log10_tau,
                         double* theta_fallback, uint32_t* count_cap, uint32_t* flags) {
    if (!path || !params_host || !log10_tau || !theta_fallback || !count_cap || !flags)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_policy_load: null argument");
    FILE* f = std::fopen(path, "r");
    if (!f) return nb::set_error(NB_ERR_INVALID_ARG, "nb_policy_load: cannot open %s", path);
    std::string line;
    double tau = 0, theta = 0, v = 0;
    uint32_t cap = 0, fl = 0, count = 0;
    const char* bad = nullptr;
    if (!read_line(f, line) || line != kMagic) bad = "not an opening-policy file";
    else if (!read_line(f, line) || line != kNetwork) bad = "unsupported network shape";
    else if (!read_line(f, line) || !parse_double(value_of(line, "log10_tau"), &tau))
        bad = "log10_tau";
    else if (!read_line(f, line) || !parse_double(value_of(line, "theta_fallback"), &theta))
        bad = "theta_fallback";
    else if (!read_line(f, line) || !parse_u32(value_of(line, "count_cap"), &cap))
        bad = "count_cap";
    else if (!read_line(f, line) || !parse_u32(value_of(line, "flags"), &fl) ||
             (fl & ~NB_POLICY_BOUND_ACCEPT))
        bad = "flags";
    else if (!read_line(f, line) || !parse_u32(value_of(line, "params"), &count) ||
             count != NB_MLP_PARAMS)
        bad = "params count";
    for (uint32_t i = 0; !bad && i < count; ++i) {
        if (!read_line(f, line) || !parse_double(line.c_str(), &v)) bad = "parameter value";
        else params_host[i] = (float)v;
    }
    std::fclose(f);
    if (bad)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_policy_load: %s: bad or missing %s", path,
                             bad);
    *log10_tau = (float)tau;
    *theta_fallback = theta;
    *count_cap = cap;
    *flags = fl;
    return NB_OK;
}

}  // extern "C"
