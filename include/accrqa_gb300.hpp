// accrqa_gb300.hpp -- the C++ API of libaccrqa.so: the overload set of the
// AccRQA reference's public header (include/AccRQA_functions.hpp:23-445),
// same names, parameter lists, output layouts and error convention, so that
// C++ callers of the reference relink against this library unchanged.
//
// Output layouts (slowest to fastest index):
//   accrqa_RR : [nTaus][nEmbs][nThresholds]
//   accrqa_DET: [nTaus][nEmbs][nLmins][nThresholds][5] = {DET, L, Lmax, ENTR, RR}
//   accrqa_LAM: [nTaus][nEmbs][nVmins][nThresholds][5] = {LAM, TT, TTmax, ENTR, RR}
//   accrqa_RP : [nc][nc] row-major, nc = data_size - (emb-1)*tau
//
// Platform: comp_platform = PLT_NV_GPU runs on the GB300.  This library has
// no CPU implementation: PLT_CPU and unknown platforms return
// ERR_INVALID_ARGUMENT with a message (the reference's own library serves the
// CPU platform).  Without a usable CUDA device the calls return
// ERR_CUDA_DEVICE_NOT_FOUND; there is no silent fallback.
//
// DET/LAM select their output convention as the reference's GPU dispatch
// does (src/AccRQA_functions.cpp:499-506,754-761): with calc_ENTR == 1 or
// max(lmin) >= 16 all five measures come from the full histogram; otherwise
// Lmax/TTmax and ENTR are NaN and RR is normalised by (nc-1)^2, as the
// reference's boxcar kernels report it (src/AccRQA-GPU-HST.cu:2438-2449,
// :2626-2636).  DET/L and LAM/TT are the same in both conventions.
#ifndef ACCRQA_GB300_HPP
#define ACCRQA_GB300_HPP

#include <cstddef>
#include <cstdint>

#include "accrqa_gb300.h"

// include/AccRQA_functions.hpp:25
void accrqa_print_error(Accrqa_Error *error);

// include/AccRQA_functions.hpp:77-86 / :121-130
void accrqa_LAM(float *output, float *input_data, size_t data_size,
                int *tau_values, int nTaus, int *emb_values, int nEmbs,
                int *vmin_values, int nVmins, float *threshold_values,
                int nThresholds, Accrqa_Distance distance_type, int calc_ENTR,
                Accrqa_CompPlatform comp_platform, Accrqa_Error *error);
void accrqa_LAM(double *output, double *input_data, size_t data_size,
                int *tau_values, int nTaus, int *emb_values, int nEmbs,
                int *vmin_values, int nVmins, double *threshold_values,
                int nThresholds, Accrqa_Distance distance_type, int calc_ENTR,
                Accrqa_CompPlatform comp_platform, Accrqa_Error *error);
// include/AccRQA_functions.hpp:141-143
int accrqa_LAM_output_size_in_elements(int nTaus, int nEmbs, int nVmins,
                                       int nThresholds);

// include/AccRQA_functions.hpp:191-200 / :235-244
void accrqa_DET(float *output, float *input_data, size_t data_size,
                int *tau_values, int nTaus, int *emb_values, int nEmbs,
                int *lmin_values, int nLmins, float *threshold_values,
                int nThresholds, Accrqa_Distance distance_type, int calc_ENTR,
                Accrqa_CompPlatform comp_platform, Accrqa_Error *error);
void accrqa_DET(double *output, double *input_data, size_t data_size,
                int *tau_values, int nTaus, int *emb_values, int nEmbs,
                int *lmin_values, int nLmins, double *threshold_values,
                int nThresholds, Accrqa_Distance distance_type, int calc_ENTR,
                Accrqa_CompPlatform comp_platform, Accrqa_Error *error);
// include/AccRQA_functions.hpp:255-257
int accrqa_DET_output_size_in_elements(int nTaus, int nEmbs, int nLmins,
                                       int nThresholds);

// include/AccRQA_functions.hpp:299-306 / :337-344
void accrqa_RR(float *output, float *input_data, size_t data_size,
               int *tau_values, int nTaus, int *emb_values, int nEmbs,
               float *threshold_values, int nThresholds,
               Accrqa_Distance distance_type, Accrqa_CompPlatform comp_platform,
               Accrqa_Error *error);
void accrqa_RR(double *output, double *input_data, size_t data_size,
               int *tau_values, int nTaus, int *emb_values, int nEmbs,
               double *threshold_values, int nThresholds,
               Accrqa_Distance distance_type, Accrqa_CompPlatform comp_platform,
               Accrqa_Error *error);
// include/AccRQA_functions.hpp:354-356
int accrqa_RR_output_size_in_elements(int nTaus, int nEmbs, int nThresholds);

// include/AccRQA_functions.hpp:383-391 / :416-424 / :427-435.  Like the
// reference, RP returns at once when *error is not SUCCESS on entry.
void accrqa_RP(char *output, float *input_data, size_t data_size, int tau,
               int emb, float threshold, Accrqa_Distance distance_type,
               Accrqa_Error *error);
void accrqa_RP(char *output, double *input_data, size_t data_size, int tau,
               int emb, double threshold, Accrqa_Distance distance_type,
               Accrqa_Error *error);
void accrqa_RP(int *output, double *input_data, size_t data_size, int tau,
               int emb, double threshold, Accrqa_Distance distance_type,
               Accrqa_Error *error);
// include/AccRQA_functions.hpp:445-447.  Returns nc (not nc*nc), as the
// reference does (src/AccRQA_functions.cpp:989-994).
int64_t accrqa_RP_output_size_in_elements(int64_t input_size, int64_t tau,
                                          int64_t emb);

#endif  // ACCRQA_GB300_HPP
