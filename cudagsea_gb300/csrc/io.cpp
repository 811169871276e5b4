// io.cpp -- Broad file formats (GCT / CLS / GMT) and the reference's loader
// proxies.
//
// Follows read_gct / read_gmt / read_cls (src/include/read_data_files.cuh:46-321)
// and the loader proxies (src/cudaGSEA_wrapper.cu:43-81): same parsing rules,
// same trimming of symbols, same checks -- but every failure throws
// std::runtime_error with the reference's message instead of exit(code):
//   GCT  first line must be "#1.2"; dimensions on line 2; a NAME/DESCRIPTION
//        header with the patient names; one row per gene: symbol (trimmed),
//        description (ignored), one value per patient; duplicate symbols are
//        an error.  Values are returned gene-major, as read.
//   CLS  "<patients> <classes> 1" with exactly two classes; "# <name0>
//        <name1>"; one label per patient, symbolic or 0/1.
//   GMT  one set per line: name, description (ignored), trimmed symbols.
#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/gsea103.h"
#include "../../include/gsea103_proxy.hpp"

namespace gsea {
void set_last_error(const char* msg);  // capi.cu

std::string& trim(std::string& s) {
    auto notspace = [](unsigned char c) { return !std::isspace(c); };
    s.erase(s.begin(), std::find_if(s.begin(), s.end(), notspace));
    s.erase(std::find_if(s.rbegin(), s.rend(), notspace).base(), s.end());
    return s;
}

template <class V>
void read_gct(const std::string& filename, std::vector<V>& exprs, std::vector<std::string>& plist,
              std::vector<std::string>& gsymb) {
    std::ifstream f(filename);
    if (!f.is_open()) throw std::runtime_error("Error: Unable to open file " + filename);
    std::string token;
    std::getline(f, token);
    if (trim(token) != "#1.2")
        throw std::runtime_error("Error: First line of " + filename + " is not a valid gct header");
    long long G = -1, S = -1;
    f >> G >> S;
    if (!f || G < 1 || S < 1) throw std::runtime_error("Error: invalid gct dimensions in " + filename);
    exprs.assign((size_t)G * S, V(0));
    plist.assign((size_t)S, "");
    gsymb.assign((size_t)G, "");
    std::getline(f, token, '\t');  // NAME (after the dimension line's newline)
    std::getline(f, token, '\t');  // DESCRIPTION
    for (long long p = 0; p < S - 1; p++) std::getline(f, plist[p], '\t');
    std::getline(f, plist[S - 1], '\n');
    for (auto& p : plist) trim(p);
    std::unordered_set<std::string> seen;
    for (long long g = 0; g < G; g++) {
        std::getline(f, token, '\t');
        gsymb[g] = trim(token);
        std::getline(f, token, '\t');  // description
        if (!seen.insert(gsymb[g]).second)
            throw std::runtime_error("Error: duplicate symbol " + gsymb[g]);
        for (long long p = 0; p < S; p++) {
            V v;
            if (!(f >> v)) throw std::runtime_error("Error: gct file " + filename + " ends early");
            exprs[(size_t)g * S + p] = v;
        }
    }
}

void read_cls(const std::string& filename, std::vector<uint8_t>& labels) {
    std::ifstream f(filename);
    if (!f.is_open()) throw std::runtime_error("Error: Unable to open file " + filename);
    std::string line;
    std::getline(f, line);
    std::stringstream ss(line);
    long long n = 0, classes = 0, one = 0;
    ss >> n >> classes >> one;
    if (classes != 2)
        throw std::runtime_error("ERROR: Number of phenotype classes specified in the corresponding cls file " +
                                 filename + " must be exactly two");
    if (one != 1) throw std::runtime_error("ERROR: Invalid header found in the corresponding cls file " + filename);
    std::getline(f, line);
    std::string names = line.substr(line.find('#') == std::string::npos ? 0 : line.find('#') + 1);
    std::stringstream ns(names);
    std::string c0, c1;
    ns >> c0;
    std::getline(ns, c1);
    trim(c0);
    trim(c1);
    std::getline(f, line);
    std::stringstream ls(line);
    labels.assign((size_t)n, 0);
    for (long long i = 0; i < n; i++) {
        std::string x;
        ls >> x;
        if (!c0.empty() && x == c0) labels[i] = 0;
        else if (!c1.empty() && x == c1) labels[i] = 1;
        else if (x == "0") labels[i] = 0;
        else if (x == "1") labels[i] = 1;
        else throw std::runtime_error("ERROR: Unknown label in cls file " + filename + " : \"" + x + "\"");
    }
}

void read_gmt(const std::string& filename, std::vector<std::string>& names,
              std::vector<std::vector<std::string>>& sets) {
    std::ifstream f(filename);
    if (!f.is_open()) throw std::runtime_error("Error: Unable to open file " + filename);
    names.clear();
    sets.clear();
    std::string line, token;
    while (std::getline(f, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::stringstream ss(line);
        std::getline(ss, token, '\t');
        names.push_back(token);
        std::vector<std::string> symbols;
        size_t count = 0;
        while (std::getline(ss, token, '\t'))
            if (count++) symbols.push_back(trim(token));
        sets.push_back(std::move(symbols));
    }
}

template void read_gct<float>(const std::string&, std::vector<float>&, std::vector<std::string>&,
                              std::vector<std::string>&);
template void read_gct<double>(const std::string&, std::vector<double>&, std::vector<std::string>&,
                               std::vector<std::string>&);

}  // namespace gsea

// ---- the reference's loader proxies (src/cudaGSEA_wrapper.cuh:15-25)
void loadLabelsFromCLS_proxy(std::string cls, std::vector<proxy_label_t>& labels) {
    std::vector<uint8_t> l;
    gsea::read_cls(cls, l);
    labels.assign(l.begin(), l.end());
}

void loadGeneSetsFromGMT_proxy(std::string gmt, std::vector<proxy_strng_t>& names,
                               std::vector<std::vector<proxy_strng_t>>& sets) {
    gsea::read_gmt(gmt, names, sets);
}

void loadExpressionDataFromGCT_proxy(std::string gct, std::vector<proxy_value_t>& exprs,
                                     std::vector<proxy_strng_t>& symbols, std::vector<proxy_strng_t>& patients) {
    gsea::read_gct<proxy_value_t>(gct, exprs, patients, symbols);
}

// ---- data sets for C callers: the three files parsed and mapped to arrays
struct gsea_dataset_s {
    std::vector<double> exprs_gm;   // gene-major, as read, parsed as double
    std::vector<float> exprs_gm_f;  // the same values parsed directly as float (as the
                                    // reference's single-precision reader does)
    std::vector<std::string> genes, patients, set_names;
    std::vector<std::vector<std::string>> sets;
    std::vector<uint8_t> labels;
    std::vector<int64_t> off;
    std::vector<int32_t> members;
};

extern "C" int gsea_dataset_load(const char* gct, const char* cls, const char* gmt, gsea_dataset* out) {
    if (!gct || !cls || !gmt || !out) {
        gsea::set_last_error("null argument");
        return GSEA_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    try {
        auto* d = new gsea_dataset_s();
        try {
            gsea::read_gct<double>(gct, d->exprs_gm, d->patients, d->genes);
            std::vector<std::string> p2, g2;
            gsea::read_gct<float>(gct, d->exprs_gm_f, p2, g2);
            gsea::read_cls(cls, d->labels);
            gsea::read_gmt(gmt, d->set_names, d->sets);
        } catch (...) {
            delete d;
            throw;
        }
        if (d->labels.size() != d->patients.size()) {
            delete d;
            throw std::runtime_error("ERROR: Incompatible class file (cls) and expression data file");
        }
        // symbol -> gene index, unknown symbols dropped, duplicates collapsed
        std::unordered_map<std::string, int32_t> index;
        for (size_t g = 0; g < d->genes.size(); g++) index.emplace(d->genes[g], (int32_t)g);
        d->off.assign(d->sets.size() + 1, 0);
        std::vector<int32_t> tmp;
        for (size_t k = 0; k < d->sets.size(); k++) {
            tmp.clear();
            for (const auto& s : d->sets[k]) {
                auto it = index.find(s);
                if (it != index.end()) tmp.push_back(it->second);
            }
            std::sort(tmp.begin(), tmp.end());
            tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
            d->members.insert(d->members.end(), tmp.begin(), tmp.end());
            d->off[k + 1] = (int64_t)d->members.size();
        }
        *out = d;
        return GSEA_OK;
    } catch (const std::exception& e) {
        gsea::set_last_error(e.what());
        return GSEA_ERR_IO;
    }
}

extern "C" int gsea_dataset_dims(gsea_dataset d, int64_t* genes, int64_t* samples, int64_t* sets,
                                 int64_t* members) {
    if (!d) {
        gsea::set_last_error("null data set");
        return GSEA_ERR_INVALID_ARGUMENT;
    }
    if (genes) *genes = (int64_t)d->genes.size();
    if (samples) *samples = (int64_t)d->patients.size();
    if (sets) *sets = (int64_t)d->sets.size();
    if (members) *members = (int64_t)d->members.size();
    return GSEA_OK;
}

extern "C" int gsea_dataset_arrays(gsea_dataset d, int precision, void* exprs_pm, uint8_t* labels,
                                   int64_t* set_offsets, int32_t* set_genes) {
    if (!d || (precision != 32 && precision != 64)) {
        gsea::set_last_error("invalid arguments");
        return GSEA_ERR_INVALID_ARGUMENT;
    }
    const size_t G = d->genes.size(), S = d->patients.size();
    if (exprs_pm) {  // transpose gene-major -> patient-major
        for (size_t g = 0; g < G; g++)
            for (size_t s = 0; s < S; s++) {
                if (precision == 64) static_cast<double*>(exprs_pm)[s * G + g] = d->exprs_gm[g * S + s];
                else static_cast<float*>(exprs_pm)[s * G + g] = d->exprs_gm_f[g * S + s];
            }
    }
    if (labels) std::copy(d->labels.begin(), d->labels.end(), labels);
    if (set_offsets) std::copy(d->off.begin(), d->off.end(), set_offsets);
    if (set_genes) std::copy(d->members.begin(), d->members.end(), set_genes);
    return GSEA_OK;
}

extern "C" const char* gsea_dataset_gene(gsea_dataset d, int64_t i) {
    return (d && i >= 0 && (size_t)i < d->genes.size()) ? d->genes[i].c_str() : nullptr;
}

extern "C" const char* gsea_dataset_set_name(gsea_dataset d, int64_t k) {
    return (d && k >= 0 && (size_t)k < d->set_names.size()) ? d->set_names[k].c_str() : nullptr;
}

extern "C" void gsea_dataset_free(gsea_dataset d) { delete d; }
