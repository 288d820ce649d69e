// host_struct.h -- the last step of loop1, shared by the host version
// (mpgpu_host_labels, host_pede.cpp) and the device version
// (mpgpu_loop1_device, mpgpu_struct.cu) so that both give identical tables.
#pragma once
#include <cstdint>
#include <vector>

// From the sorted distinct labels `all` and, per label, the entries `cnt`,
// the group cut after it `cut[i]` (between i and i+1) and whether a
// non-zero derivative met it `seen`: pre-sigmas, the entries cut
// (pede.f90:5958-5971), the variable numbering and the parameter groups
// (pede.f90:2311-2404, 6509-6545).  Writes the output tables of
// mpgpu_host_labels and returns the number of labels.
int32_t labels_finish(const std::vector<int32_t> &all, const std::vector<int64_t> &cnt,
                      const std::vector<uint8_t> &cut, const std::vector<uint8_t> &seen, int32_t npre,
                      const int32_t *preLabel, const double *preSigma, int32_t mreqenf, int32_t *labels,
                      int64_t *counter, int32_t *varIndex, int32_t *totGroup, int32_t *nVar,
                      int32_t *nVarGroups);
