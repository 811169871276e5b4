// gsea103_proxy.hpp -- C++ proxy API of libgsea103, source-compatible with
// cudaGSEA's R bridge (src/cudaGSEA_wrapper.cuh:1-61): an Rcpp layer written
// against the reference links against libgsea103.so unchanged.
//
// Differences from the reference: errors throw std::runtime_error (which Rcpp
// turns into an R error) instead of calling exit(); the fifth block of the
// returned statistics holds FDR q-values instead of NaN.
#pragma once
#include <cstddef>
#include <string>
#include <vector>

// fixed data types for the communication with R (src/cudaGSEA_wrapper.cuh:6-9)
typedef std::string proxy_strng_t;
typedef double proxy_value_t;
typedef size_t proxy_label_t;
typedef size_t proxy_index_t;

// Broad file formats (src/cudaGSEA_wrapper.cuh:15-25, readers
// src/include/read_data_files.cuh:46-321)
void loadLabelsFromCLS_proxy(std::string, std::vector<proxy_label_t>&);
void loadGeneSetsFromGMT_proxy(std::string, std::vector<proxy_strng_t>&,
                               std::vector<std::vector<proxy_strng_t>>&);
void loadExpressionDataFromGCT_proxy(std::string, std::vector<proxy_value_t>&,
                                     std::vector<proxy_strng_t>&, std::vector<proxy_strng_t>&);

// CUDA device control (src/cudaGSEA_wrapper.cuh:31-33)
std::vector<proxy_strng_t> listCudaDevices_proxy();
int getCudaDevice_proxy();
int setCudaDevice_proxy(int);

// GSEA (src/cudaGSEA_wrapper.cuh:39-61, definitions src/cudaGSEA_wrapper.cu:403-437)
//   exprs  patient-major: exprs[patient * gsymb.size() + gene]
//   labels 0/1 per patient (swapped in place when swap_labels is true)
//   result struct of arrays [ES | NES | NP | FWER | FDR], pathw.size() each
std::vector<float> gsea_single_proxy(std::vector<float>& exprs, std::vector<std::string>& gsymb,
                                     std::vector<std::string>& plist, std::vector<char>& labels,
                                     std::vector<std::string>& pname,
                                     std::vector<std::vector<std::string>>& pathw,
                                     std::string metric, size_t num_perms, bool sort_direction,
                                     bool swap_labels, std::string dump_filename);

std::vector<double> gsea_double_proxy(std::vector<double>& exprs, std::vector<std::string>& gsymb,
                                      std::vector<std::string>& plist, std::vector<char>& labels,
                                      std::vector<std::string>& pname,
                                      std::vector<std::vector<std::string>>& pathw,
                                      std::string metric, size_t num_perms, bool sort_direction,
                                      bool swap_labels, std::string dump_filename);
