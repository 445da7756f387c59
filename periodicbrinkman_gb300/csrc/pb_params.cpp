// Parameter files in the format of the reference's driver: text lines whose
// first token is a parameter name and whose second token is its value,
// tokens separated by any of the delimiter characters (default ": "), read
// as readData does (cuda/periodicBrinkman.cu:44-70 for the name -> value map,
// cuda/periodicBrinkman.h:524-554 for the array twin over given names).
// Values convert as atof does (a non-numeric value reads as 0).  Unlike the
// reference: lines may be of any length (its 80-byte line buffer stops
// reading at a longer line), and a line with a name but no value is an
// error (the reference passes a null pointer to atof there).
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "pb_internal.h"
#include "pbrinkman.h"

namespace {

// The first two tokens of `line` split at any character of `delims` (the
// strtok rule: runs of delimiters separate, leading ones are skipped).
int tokens(const std::string& line, const char* delims, std::string& key, std::string& value)
{
    auto is_delim = [&](char c) { return c != '\0' && std::strchr(delims, c) != nullptr; };
    size_t i = 0, n = line.size();
    while (i < n && is_delim(line[i])) i++;
    if (i >= n) return 0;
    size_t k0 = i;
    while (i < n && !is_delim(line[i])) i++;
    key.assign(line, k0, i - k0);
    while (i < n && is_delim(line[i])) i++;
    if (i >= n) return 1;
    size_t v0 = i;
    while (i < n && !is_delim(line[i])) i++;
    value.assign(line, v0, i - v0);
    return 2;
}

// Reads every (name, value) line; calls put(name, value) in file order.
template <class Put>
int read_lines(const char* file_name, const char* delimiters, Put put)
{
    if (!file_name) return pb::api_error(PB_ERR_INVALID, "null file name");
    const char* delims = delimiters ? delimiters : ": ";
    std::ifstream in(file_name);
    if (!in.good()) return pb::api_error(PB_ERR_INVALID, "cannot open the parameter file");
    std::string line, key, value;
    int lineno = 0;
    while (std::getline(in, line)) {
        lineno++;
        if (!line.empty() && line.back() == '\r') line.pop_back();
        const int nt = tokens(line, delims, key, value);
        if (nt == 0) continue;
        if (nt == 1) {
            std::string msg = "parameter file line " + std::to_string(lineno) + ": name without a value";
            return pb::api_error(PB_ERR_INVALID, msg.c_str());
        }
        int rc = put(key, std::atof(value.c_str()));
        if (rc) return rc;
    }
    return PB_OK;
}

}  // namespace

extern "C" int pb_read_params(const char* file_name, const char* delimiters, const char* const* names,
                              double* values, int numel)
{
    if (numel < 0 || (numel > 0 && (!names || !values))) return pb::api_error(PB_ERR_INVALID, "bad arguments");
    return read_lines(file_name, delimiters, [&](const std::string& key, double v) {
        for (int n = 0; n < numel; n++)
            if (names[n] && key == names[n]) {
                values[n] = v;
                break;
            }
        return 0;
    });
}

extern "C" int pb_read_param_file(const char* file_name, const char* delimiters, char (*keys)[64], double* values,
                                  int max_keys)
{
    if (max_keys < 0 || (max_keys > 0 && (!keys || !values))) return pb::api_error(PB_ERR_INVALID, "bad arguments");
    std::vector<std::string> names;
    std::vector<double> vals;
    int rc = read_lines(file_name, delimiters, [&](const std::string& key, double v) {
        if (key.size() > 63) return pb::api_error(PB_ERR_UNSUPPORTED, "parameter name longer than 63 characters");
        for (size_t k = 0; k < names.size(); k++)
            if (names[k] == key) {
                vals[k] = v;  // a later line overrides, as assigning the map entry does
                return 0;
            }
        names.push_back(key);
        vals.push_back(v);
        return 0;
    });
    if (rc) return rc;
    for (size_t k = 0; k < names.size() && (int)k < max_keys; k++) {
        std::memcpy(keys[k], names[k].c_str(), names[k].size() + 1);
        values[k] = vals[k];
    }
    return (int)names.size();
}
