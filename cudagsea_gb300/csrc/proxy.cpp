// proxy.cpp -- the reference's C++ proxy API (include/gsea103_proxy.hpp) on
// top of the C ABI, plus a flat C entry point with the same semantics for
// foreign-function callers (ctypes, cgo, JNI) that cannot pass std::vector.
//
// gsea_proxy<> (src/cudaGSEA_wrapper.cu:179-401) maps gene-set symbols to gene
// indices by building one bitmap per 32/64-set batch on the host inside every
// permutation batch (create_bitmaps.cuh:13-65).  Here symbols are mapped once,
// on the device (gsea_map_sets: hash table of the gene symbols, per-set
// membership bitmasks, CSR): unknown symbols are dropped and duplicates
// collapse, which is exactly the membership the bitmaps encode.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gsea103.h"
#include "../../include/gsea103_proxy.hpp"

namespace gsea {
void set_last_error(const char* msg);  // capi.cu
}

namespace {

// a failed C-ABI call, with its status
struct status_error : std::runtime_error {
    int status;
    status_error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

struct Csr {
    std::vector<int64_t> off;
    std::vector<int32_t> genes;
};

// symbols -> CSR of gene indices on the device (gsea_map_sets, csrc/sets.cu)
Csr map_sets(const std::vector<std::string>& gsymb, const std::vector<std::vector<std::string>>& pathw) {
    if (gsymb.empty()) throw status_error(GSEA_ERR_INVALID_ARGUMENT, "empty expression table");
    std::vector<const char*> gp(gsymb.size());
    for (size_t g = 0; g < gsymb.size(); g++) gp[g] = gsymb[g].c_str();
    std::vector<int64_t> soff(pathw.size() + 1, 0);
    std::vector<const char*> sp;
    for (size_t k = 0; k < pathw.size(); k++) {
        for (const auto& m : pathw[k]) sp.push_back(m.c_str());
        soff[k + 1] = (int64_t)sp.size();
    }
    Csr c;
    c.off.resize(pathw.size() + 1, 0);
    c.genes.resize(sp.size());
    int64_t nnz = 0;
    const int rc = gsea_map_sets((int64_t)gp.size(), gp.data(), (int64_t)pathw.size(), soff.data(), sp.data(),
                                 c.off.data(), c.genes.data(), (int64_t)sp.size(), &nnz);
    if (rc) throw status_error(rc, gsea_last_error());
    c.genes.resize((size_t)nnz);
    return c;
}

template <class T>
std::vector<T> run_proxy(std::vector<T>& exprs, std::vector<std::string>& gsymb, std::vector<std::string>& plist,
                         std::vector<char>& labels, std::vector<std::string>& pname,
                         std::vector<std::vector<std::string>>& pathw, const std::string& metric,
                         size_t num_perms, bool sort_direction, bool swap_labels,
                         const std::string& dump_filename) {
    const int64_t G = (int64_t)gsymb.size(), S = (int64_t)plist.size(), K = (int64_t)pname.size();
    if ((int64_t)pathw.size() != K)
        throw status_error(GSEA_ERR_INVALID_ARGUMENT, "gene set names and gene sets differ in length");
    if ((int64_t)exprs.size() != G * S)
        throw status_error(GSEA_ERR_INVALID_ARGUMENT, "expression table is not genes x patients");
    if ((int64_t)labels.size() != S)
        throw status_error(GSEA_ERR_INVALID_ARGUMENT, "label list length differs from patient count");
    const int mid = gsea_metric_id(metric.c_str());
    if (mid < 0) throw status_error(GSEA_ERR_UNKNOWN_METRIC, "unknown metric: " + metric);
    // swap_labels flips the caller's labels in place (cudaGSEA_wrapper.cu:246-251)
    if (swap_labels)
        for (auto& l : labels) l = (char)((l + 1) & 1);
    std::vector<uint8_t> lab(labels.begin(), labels.end());
    Csr sets = map_sets(gsymb, pathw);
    gsea_config cfg;
    gsea_config_init(&cfg);
    cfg.num_genes = G;
    cfg.num_samples = S;
    cfg.num_sets = K;
    cfg.num_perms = (int64_t)num_perms;
    cfg.metric = mid;
    cfg.precision = sizeof(T) == 8 ? 64 : 32;
    cfg.ascending = sort_direction ? 0 : 1;
    std::vector<T> result(5 * (size_t)K);
    const int rc = gsea_run(&cfg, exprs.data(), lab.data(), sets.off.data(), sets.genes.data(), nullptr,
                            result.data(), dump_filename.empty() ? nullptr : dump_filename.c_str());
    if (rc != GSEA_OK)
        throw status_error(rc, std::string("GSEA failed: ") + gsea_status_string(rc) + ": " + gsea_last_error());
    return result;
}

}  // namespace

std::vector<float> gsea_single_proxy(std::vector<float>& exprs, std::vector<std::string>& gsymb,
                                     std::vector<std::string>& plist, std::vector<char>& labels,
                                     std::vector<std::string>& pname, std::vector<std::vector<std::string>>& pathw,
                                     std::string metric, size_t num_perms, bool sort_direction, bool swap_labels,
                                     std::string dump_filename) {
    return run_proxy<float>(exprs, gsymb, plist, labels, pname, pathw, metric, num_perms, sort_direction,
                            swap_labels, dump_filename);
}

std::vector<double> gsea_double_proxy(std::vector<double>& exprs, std::vector<std::string>& gsymb,
                                      std::vector<std::string>& plist, std::vector<char>& labels,
                                      std::vector<std::string>& pname, std::vector<std::vector<std::string>>& pathw,
                                      std::string metric, size_t num_perms, bool sort_direction, bool swap_labels,
                                      std::string dump_filename) {
    return run_proxy<double>(exprs, gsymb, plist, labels, pname, pathw, metric, num_perms, sort_direction,
                             swap_labels, dump_filename);
}

std::vector<proxy_strng_t> listCudaDevices_proxy() {
    int n = 0;
    if (gsea_device_count(&n) != GSEA_OK) throw std::runtime_error(gsea_last_error());
    std::vector<proxy_strng_t> out;
    char buf[512];
    for (int d = 0; d < n; d++) {
        if (gsea_device_string(d, buf, sizeof(buf)) != GSEA_OK) throw std::runtime_error(gsea_last_error());
        out.emplace_back(buf);
    }
    return out;
}

int getCudaDevice_proxy() {
    int d = 0;
    if (gsea_get_device(&d) != GSEA_OK) throw std::runtime_error(gsea_last_error());
    return d;
}

int setCudaDevice_proxy(int id) {
    int active = 0;
    gsea_set_device(id, &active);  // falls back to the current device on an invalid id
    return active;
}

// ---------------------------------------------------------------------------
// flat C entry point with the proxy's semantics
extern "C" int gsea_proxy_run(int precision, const void* exprs, int64_t num_genes, int64_t num_samples,
                              const char* const* gene_symbols, const uint8_t* labels, int64_t num_sets,
                              const int64_t* set_symbol_offsets, const char* const* set_symbols,
                              const char* metric, int64_t num_perms, int sort_direction, int swap_labels,
                              const char* dump_filename, void* result_out) {
    try {
        std::vector<std::string> gsymb(gene_symbols, gene_symbols + num_genes);
        std::vector<std::string> plist((size_t)num_samples);
        for (int64_t s = 0; s < num_samples; s++) plist[s] = "p" + std::to_string(s);
        std::vector<char> lab(labels, labels + num_samples);
        std::vector<std::string> pname((size_t)num_sets);
        std::vector<std::vector<std::string>> pathw((size_t)num_sets);
        for (int64_t k = 0; k < num_sets; k++) {
            pname[k] = std::to_string(k + 1);
            for (int64_t i = set_symbol_offsets[k]; i < set_symbol_offsets[k + 1]; i++)
                pathw[k].emplace_back(set_symbols[i]);
        }
        const std::string dump = dump_filename ? dump_filename : "";
        if (precision == 64) {
            const double* x = static_cast<const double*>(exprs);
            std::vector<double> ex(x, x + num_genes * num_samples);
            auto r = gsea_double_proxy(ex, gsymb, plist, lab, pname, pathw, metric ? metric : "",
                                       (size_t)num_perms, sort_direction != 0, swap_labels != 0, dump);
            std::memcpy(result_out, r.data(), r.size() * sizeof(double));
        } else {
            const float* x = static_cast<const float*>(exprs);
            std::vector<float> ex(x, x + num_genes * num_samples);
            auto r = gsea_single_proxy(ex, gsymb, plist, lab, pname, pathw, metric ? metric : "",
                                       (size_t)num_perms, sort_direction != 0, swap_labels != 0, dump);
            std::memcpy(result_out, r.data(), r.size() * sizeof(float));
        }
        return GSEA_OK;
    } catch (const status_error& e) {
        gsea::set_last_error(e.what());
        return e.status;
    } catch (const std::exception& e) {
        gsea::set_last_error(e.what());
        return GSEA_ERR_INVALID_ARGUMENT;
    }
}
