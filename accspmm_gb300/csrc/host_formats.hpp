// host_formats.hpp -- host-side builders (host_formats.cpp).
#pragma once

#include <cstdint>
#include <vector>

#include "accspmm.h"

namespace accspmm {

int read_mtx_host(const char* path, accspmm_coo_t* coo);
int csr_from_coo_host(const accspmm_coo_t* coo, accspmm_csr_t* csr);
int metcf_from_csr_host(const accspmm_csr_t* csr, accspmm_metcf_t* out);
std::vector<uint32_t> adp_groups_host(uint32_t W, const uint32_t* rwo, uint32_t t_load,
                                      uint32_t t_comp, uint32_t t_write, uint32_t target_num);
int adpbme_from_metcf_host(const accspmm_metcf_t* m, uint32_t t_load, uint32_t t_comp,
                           uint32_t t_write, uint32_t target_num, accspmm_adpbme_t* a);
int balance_strategy_host(const uint32_t* rwo, uint32_t W, uint32_t T);

// binary files (metcf_io.cpp)
int metcf_save(const accspmm_metcf_t* m, const char* path, void* stream);
int metcf_load(const char* path, int32_t space, accspmm_metcf_t* out, void* stream);
int adpbme_save(const accspmm_adpbme_t* a, const char* path, void* stream);
int adpbme_load(const char* path, int32_t space, accspmm_adpbme_t* out, void* stream);

// locality reordering (reorder.cpp)
int reorder_rcm_host(const accspmm_csr_t* a, uint32_t* perm, uint64_t* bw_before, uint64_t* bw_after);
int csr_permute_host(const accspmm_csr_t* a, const uint32_t* perm, accspmm_csr_t* out);

// device builders (metcf_device.cu)
int csr_from_coo_device(const accspmm_coo_t* coo, accspmm_csr_t* csr, void* stream);
int metcf_from_csr_device(const accspmm_csr_t* csr, accspmm_metcf_t* out, void* stream);
int adpbme_from_metcf_device(const accspmm_metcf_t* m, uint32_t t_load, uint32_t t_comp,
                             uint32_t t_write, uint32_t target_num, accspmm_adpbme_t* a,
                             void* stream);
int balance_strategy_device(const accspmm_metcf_t* m, int* adaptive, void* stream);

}  // namespace accspmm
