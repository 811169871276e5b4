// cli.cpp -- `gsea103`, the command-line front end of libgsea103.
//
// Mirrors the reference CLI (src/cudaGSEA.cu:8-191, src/HELP.txt): the same
// flags, defaults (16,384 permutations, onepass_signal2noise, descending,
// single precision, GPU 0) and the same "RESULT:" lines
// (src/include/cugsea.cuh:437-444).  The reference's -cpu mode has no
// counterpart: all compute runs on the GPU; -form selects the plain or the
// tensor-core form.  Exit codes follow src/include/error_codes.cuh.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/gsea103.h"

namespace {

const char* arg(int argc, char** argv, const char* flag) {
    for (int i = 1; i + 1 < argc; i++)
        if (std::strcmp(argv[i], flag) == 0) return argv[i + 1];
    return nullptr;
}
bool has(int argc, char** argv, const char* flag) {
    for (int i = 1; i < argc; i++)
        if (std::strcmp(argv[i], flag) == 0) return true;
    return false;
}
bool is_number(const char* s) {
    if (!s || !*s) return false;
    for (const char* c = s; *c; c++)
        if (*c < '0' || *c > '9') return false;
    return true;
}

void help() {
    std::cout << "INFO: gsea103 -res <file.gct> -cls <file.cls> -gmx <file.gmt>\n"
                 "INFO:        [-nperm <16384>] [-metric <onepass_signal2noise>]\n"
                 "INFO:        [-order ascending|<descending>] [-dump <prefix>]\n"
                 "INFO:        [-precision <single>|double] [-gpu <0>] [-form <plain>|chosen]\n";
}

template <class T>
int run(gsea_dataset ds, gsea_config& cfg, const std::string& dump) {
    int64_t G, S, K, nnz;
    gsea_dataset_dims(ds, &G, &S, &K, &nnz);
    std::vector<T> x((size_t)G * S);
    std::vector<uint8_t> labels((size_t)S);
    std::vector<int64_t> off((size_t)K + 1);
    std::vector<int32_t> genes((size_t)nnz > 0 ? (size_t)nnz : 1);
    gsea_dataset_arrays(ds, sizeof(T) * 8, x.data(), labels.data(), off.data(), genes.data());
    cfg.num_genes = G;
    cfg.num_samples = S;
    cfg.num_sets = K;
    std::vector<T> stats(5 * (size_t)K);
    const int rc = gsea_run(&cfg, x.data(), labels.data(), off.data(), genes.data(), nullptr, stats.data(),
                            dump.empty() ? nullptr : dump.c_str());
    if (rc) {
        std::cout << "ERROR: " << gsea_status_string(rc) << ": " << gsea_last_error() << std::endl;
        return rc == GSEA_ERR_UNKNOWN_METRIC ? 1 : 21;
    }
    for (int64_t k = 0; k < K; k++) {
        std::cout << std::showpos << std::fixed << "RESULT:"
                  << " ES: " << stats[k] << " NES: " << stats[K + k] << " NP: " << stats[2 * K + k]
                  << " FWER: " << stats[3 * K + k] << "\t(" << gsea_dataset_set_name(ds, k) << ")" << std::endl;
    }
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc == 1) {
        help();
        return 1;
    }
    const char* res = arg(argc, argv, "-res");
    const char* cls = arg(argc, argv, "-cls");
    const char* gmx = arg(argc, argv, "-gmx");
    if (!res) {
        help();
        std::cout << "ERROR: You have to specify a collapsed gene expression file with -res. Exiting." << std::endl;
        return 11;
    }
    if (!cls) {
        help();
        std::cout << "ERROR: You have to specify a class label assignment file with -cls. Exiting." << std::endl;
        return 12;
    }
    if (!gmx) {
        help();
        std::cout << "ERROR: You have to specify a gene set file with -gmx. Exiting." << std::endl;
        return 13;
    }
    gsea_config cfg;
    gsea_config_init(&cfg);
    cfg.num_perms = 1 << 14;
    if (has(argc, argv, "-nperm")) {
        const char* n = arg(argc, argv, "-nperm");
        if (!is_number(n)) {
            std::cout << "ERROR: number specified with -nperm could not be parsed as integer. Exiting." << std::endl;
            return 17;
        }
        cfg.num_perms = std::atoll(n);
    }
    std::string metric = "onepass_signal2noise";
    if (const char* m = arg(argc, argv, "-metric")) metric = m;
    cfg.metric = gsea_metric_id(metric.c_str());
    if (cfg.metric < 0) {
        std::cout << "ERROR: unknown metric, exiting." << std::endl;
        return 1;
    }
    if (const char* o = arg(argc, argv, "-order")) {
        if (!std::strcmp(o, "ascending")) cfg.ascending = 1;
        else if (std::strcmp(o, "descending")) {
            std::cout << "ERROR: option specified with -order must be either ascending or descending. Exiting."
                      << std::endl;
            return 18;
        }
    }
    std::string dump;
    if (has(argc, argv, "-dump")) {
        const char* d = arg(argc, argv, "-dump");
        if (!d || !*d) {
            std::cout << "ERROR: Parameter -dump observed but empty file name found. Exiting." << std::endl;
            return 19;
        }
        dump = d;
    }
    bool single = true;
    if (const char* p = arg(argc, argv, "-precision")) {
        if (!std::strcmp(p, "double")) single = false;
        else if (std::strcmp(p, "single")) {
            std::cout << "ERROR: option specified with -precision must be either single or double. Exiting."
                      << std::endl;
            return 20;
        }
    }
    if (has(argc, argv, "-cpu")) {
        std::cout << "ERROR: gsea103 computes on the GPU only; -cpu is not available. Exiting." << std::endl;
        return 22;
    }
    if (has(argc, argv, "-gpu")) {
        const char* g = arg(argc, argv, "-gpu");
        if (!is_number(g)) {
            std::cout << "ERROR: number specified with -gpu could not be parsed as integer. Exiting." << std::endl;
            return 17;
        }
        cfg.device = std::atoi(g);
    }
    if (const char* f = arg(argc, argv, "-form")) cfg.form = !std::strcmp(f, "chosen") ? GSEA_FORM_CHOSEN : GSEA_FORM_PLAIN;
    cfg.precision = single ? 32 : 64;
    if (!single) cfg.form = GSEA_FORM_PLAIN;
    gsea_dataset ds = nullptr;
    if (gsea_dataset_load(res, cls, gmx, &ds) != GSEA_OK) {
        std::cout << gsea_last_error() << ", exiting." << std::endl;
        return 2;
    }
    const int rc = single ? run<float>(ds, cfg, dump) : run<double>(ds, cfg, dump);
    gsea_dataset_free(ds);
    return rc;
}
