// bindings.cpp -- the reference's foreign-function shims on top of the C++
// API: py_accrqa_* (ctypes; src/AccRQA_python_bindings.cpp), R_double_accrqa_*
// (.C; src/AccRQA_R_bindings.cpp) and the thread-count functions
// (src/AccRQA_threads.cpp).  Validation order, messages' meaning and error
// codes follow the reference so that its Python and R packages behave the
// same on top of this library.
#include <cstdio>

#include "accrqa_gb300.hpp"

namespace {

void msg(const char *m) { std::printf("%s", m); }

// src/AccRQA_python_bindings.cpp:16-30
Accrqa_Distance distance_of(int v, Accrqa_Error *error) {
    if (v == 1) return DST_EUCLIDEAN;
    if (v == 2) return DST_MAXIMAL;
    msg("Error: Invalid distance type.\n");
    *error = ERR_INVALID_ARGUMENT;
    return DST_ERROR;
}

// src/AccRQA_python_bindings.cpp:39-53
Accrqa_CompPlatform platform_of(int v, Accrqa_Error *error) {
    if (v == 1) return PLT_CPU;
    if (v == 1024) return PLT_NV_GPU;
    msg("Error: Invalid computing platform.\n");
    *error = ERR_INVALID_ARGUMENT;
    return PLT_ERROR;
}

bool all_cpu(Mem *const *ms, int n) {
    for (int i = 0; i < n; i++)
        if (mem_location(ms[i]) != MEM_CPU) return false;
    return true;
}

// Shared checks of py_accrqa_DET / py_accrqa_LAM
// (src/AccRQA_python_bindings.cpp:324-388 and :469-533).
bool line_checks(Mem *out, Mem *in, Mem *taus, Mem *embs, Mem *lm, Mem *thr,
                 Accrqa_Error *error) {
    Mem *all[6] = {out, in, taus, embs, lm, thr};
    if (!all_cpu(all, 6)) {
        msg("ERROR! Data are stored in wrong destination.\n");
        *error = ERR_MEM_LOCATION;
        return false;
    }
    if (mem_type(in) != mem_type(out) || mem_type(in) != mem_type(thr)) {
        msg("ERROR! Input, output and threshold values must have the same data type.\n");
        *error = ERR_DATA_TYPE;
        return false;
    }
    if (mem_type(taus) != MEM_INT || mem_type(embs) != MEM_INT || mem_type(lm) != MEM_INT) {
        msg("ERROR! tau, emb and lmin must be integers.\n");
        *error = ERR_DATA_TYPE;
        return false;
    }
    if (mem_num_dims(taus) != 1 || mem_num_dims(embs) != 1 || mem_num_dims(lm) != 1 ||
        mem_num_dims(thr) != 1 || mem_num_dims(in) != 1) {
        msg("input, tau, emb and threshold must be one-dimensional.\n");
        *error = ERR_INVALID_ARGUMENT;
        return false;
    }
    if (mem_num_dims(out) != 5) {
        msg("output must be five-dimensional.\n");
        *error = ERR_INVALID_ARGUMENT;
        return false;
    }
    if (mem_shape_dim(in, 0) == 0 || mem_shape_dim(taus, 0) == 0 ||
        mem_shape_dim(embs, 0) == 0 || mem_shape_dim(lm, 0) == 0 ||
        mem_shape_dim(thr, 0) == 0) {
        msg("input, tau, emb and threshold number of elements must be non zero.\n");
        *error = ERR_INVALID_ARGUMENT;
        return false;
    }
    return true;
}

template <int KIND>
void py_lines(Mem *out, Mem *in, Mem *taus, Mem *embs, Mem *lm, Mem *thr, int dist_i,
              int calc_ENTR, int plt_i, Accrqa_Error *error) {
    if (!line_checks(out, in, taus, embs, lm, thr, error)) return;
    Accrqa_Distance dist = distance_of(dist_i, error);
    if (*error != SUCCESS) return;
    Accrqa_CompPlatform plt = platform_of(plt_i, error);
    if (*error != SUCCESS) return;
    int *tv = (int *)mem_data(taus);
    int nT = (int)mem_shape_dim(taus, 0);
    int *ev = (int *)mem_data(embs);
    int nE = (int)mem_shape_dim(embs, 0);
    int *lv = (int *)mem_data(lm);
    int nL = (int)mem_shape_dim(lm, 0);
    int nThr = (int)mem_shape_dim(thr, 0);
    size_t n = (size_t)mem_shape_dim(in, 0);
    if (mem_type(in) == MEM_FLOAT) {
        if (KIND == 0)
            accrqa_DET((float *)mem_data(out), (float *)mem_data(in), n, tv, nT, ev, nE, lv, nL,
                       (float *)mem_data(thr), nThr, dist, calc_ENTR, plt, error);
        else
            accrqa_LAM((float *)mem_data(out), (float *)mem_data(in), n, tv, nT, ev, nE, lv, nL,
                       (float *)mem_data(thr), nThr, dist, calc_ENTR, plt, error);
    } else if (mem_type(in) == MEM_DOUBLE) {
        if (KIND == 0)
            accrqa_DET((double *)mem_data(out), (double *)mem_data(in), n, tv, nT, ev, nE, lv,
                       nL, (double *)mem_data(thr), nThr, dist, calc_ENTR, plt, error);
        else
            accrqa_LAM((double *)mem_data(out), (double *)mem_data(in), n, tv, nT, ev, nE, lv,
                       nL, (double *)mem_data(thr), nThr, dist, calc_ENTR, plt, error);
    } else {
        msg("ERROR! Unsupported data type.\n");
        *error = ERR_DATA_TYPE;
    }
}

}  // namespace

extern "C" {

// src/AccRQA_python_bindings.cpp:78-150
void py_accrqa_RP(Mem *out, Mem *in, int32_t tau, int32_t emb, double threshold,
                  int int_distance_type, Accrqa_Error *error) {
    if (mem_location(out) != MEM_CPU || mem_location(in) != MEM_CPU) {
        msg("ERROR! Data are stored in wrong destination.\n");
        *error = ERR_MEM_LOCATION;
        return;
    }
    if (tau <= 0 || emb <= 0) {
        msg("ERROR! Values of tau and emb must be non-zero.\n");
        *error = ERR_DATA_TYPE;
        return;
    }
    if (mem_num_dims(in) != 1) {
        msg("input must be one-dimensional array.\n");
        *error = ERR_INVALID_ARGUMENT;
        return;
    }
    if (mem_num_dims(out) != 2) {
        msg("mem_output_RP must be two-dimensional.\n");
        *error = ERR_INVALID_ARGUMENT;
        return;
    }
    if (mem_shape_dim(in, 0) == 0) {
        msg("input number of elements must be non zero.\n");
        *error = ERR_INVALID_ARGUMENT;
        return;
    }
    Accrqa_Distance dist = distance_of(int_distance_type, error);
    if (*error != SUCCESS) return;
    size_t n = (size_t)mem_shape_dim(in, 0);
    char *o = (char *)mem_data(out);
    if (mem_type(in) == MEM_FLOAT) {
        accrqa_RP(o, (float *)mem_data(in), n, tau, emb, (float)threshold, dist, error);
    } else if (mem_type(in) == MEM_DOUBLE) {
        // the reference holds this threshold in a float (src/AccRQA_python_bindings.cpp:135)
        float t = (float)threshold;
        accrqa_RP(o, (double *)mem_data(in), n, tau, emb, (double)t, dist, error);
    } else {
        msg("ERROR! Unsupported data type.\n");
        *error = ERR_DATA_TYPE;
    }
}

// src/AccRQA_python_bindings.cpp:175-276
void py_accrqa_RR(Mem *out, Mem *in, Mem *taus, Mem *embs, Mem *thr, int int_distance_type,
                  int int_comp_platform, Accrqa_Error *error) {
    Mem *all[5] = {out, in, taus, embs, thr};
    if (!all_cpu(all, 5)) {
        msg("ERROR! Data are stored in wrong destination.\n");
        *error = ERR_MEM_LOCATION;
        return;
    }
    if (mem_type(in) != mem_type(out) || mem_type(in) != mem_type(thr)) {
        msg("ERROR! Input, output and threshold values must have the same data type.\n");
        *error = ERR_DATA_TYPE;
        return;
    }
    if (mem_type(taus) != MEM_INT || mem_type(embs) != MEM_INT) {
        msg("ERROR! tau and emb must be integers.\n");
        *error = ERR_DATA_TYPE;
        return;
    }
    if (mem_num_dims(taus) != 1 || mem_num_dims(embs) != 1 || mem_num_dims(thr) != 1 ||
        mem_num_dims(in) != 1) {
        msg("input, tau, emb and threshold must be one-dimensional.\n");
        *error = ERR_INVALID_ARGUMENT;
        return;
    }
    if (mem_num_dims(out) != 3) {
        msg("mem_output_RR must be three-dimensional.\n");
        *error = ERR_INVALID_ARGUMENT;
        return;
    }
    if (mem_shape_dim(in, 0) == 0 || mem_shape_dim(taus, 0) == 0 ||
        mem_shape_dim(embs, 0) == 0 || mem_shape_dim(thr, 0) == 0) {
        msg("input, tau, emb and threshold number of elements must be non zero.\n");
        *error = ERR_INVALID_ARGUMENT;
        return;
    }
    Accrqa_Distance dist = distance_of(int_distance_type, error);
    if (*error != SUCCESS) return;
    Accrqa_CompPlatform plt = platform_of(int_comp_platform, error);
    if (*error != SUCCESS) return;
    int *tv = (int *)mem_data(taus);
    int nT = (int)mem_shape_dim(taus, 0);
    int *ev = (int *)mem_data(embs);
    int nE = (int)mem_shape_dim(embs, 0);
    int nThr = (int)mem_shape_dim(thr, 0);
    size_t n = (size_t)mem_shape_dim(in, 0);
    if (mem_type(in) == MEM_FLOAT) {
        accrqa_RR((float *)mem_data(out), (float *)mem_data(in), n, tv, nT, ev, nE,
                  (float *)mem_data(thr), nThr, dist, plt, error);
    } else if (mem_type(in) == MEM_DOUBLE) {
        accrqa_RR((double *)mem_data(out), (double *)mem_data(in), n, tv, nT, ev, nE,
                  (double *)mem_data(thr), nThr, dist, plt, error);
    } else {
        msg("ERROR! Unsupported data type.\n");
        *error = ERR_DATA_TYPE;
    }
}

// src/AccRQA_python_bindings.cpp:312-424
void py_accrqa_DET(Mem *out, Mem *in, Mem *taus, Mem *embs, Mem *lmins, Mem *thr,
                   int int_distance_type, int calc_ENTR, int int_comp_platform,
                   Accrqa_Error *error) {
    py_lines<0>(out, in, taus, embs, lmins, thr, int_distance_type, calc_ENTR,
                int_comp_platform, error);
}

// src/AccRQA_python_bindings.cpp:457-569
void py_accrqa_LAM(Mem *out, Mem *in, Mem *taus, Mem *embs, Mem *vmins, Mem *thr,
                   int int_distance_type, int calc_ENTR, int int_comp_platform,
                   Accrqa_Error *error) {
    py_lines<1>(out, in, taus, embs, vmins, thr, int_distance_type, calc_ENTR,
                int_comp_platform, error);
}

// ---------------------------------------------------------------------------
// R .C() shims (src/AccRQA_R_bindings.cpp:45-246); double precision only.
// ---------------------------------------------------------------------------
void R_double_accrqa_DET(double *output, double *input, int *input_size, int *tau_values,
                         int *nTaus, int *emb_values, int *nEmbs, int *lmin_values,
                         int *nLmins, double *threshold_values, int *nThresholds,
                         int *int_distance_type, int *calc_ENTR, int *int_comp_platform) {
    Accrqa_Error error = SUCCESS;
    Accrqa_Distance dist = distance_of(int_distance_type[0], &error);
    if (error != SUCCESS) return;
    Accrqa_CompPlatform plt = platform_of(int_comp_platform[0], &error);
    if (error != SUCCESS) return;
    accrqa_DET(output, input, (size_t)input_size[0], tau_values, nTaus[0], emb_values,
               nEmbs[0], lmin_values, nLmins[0], threshold_values, nThresholds[0], dist,
               calc_ENTR[0], plt, &error);
}

void R_double_accrqa_LAM(double *output, double *input, int *input_size, int *tau_values,
                         int *nTaus, int *emb_values, int *nEmbs, int *vmin_values,
                         int *nVmins, double *threshold_values, int *nThresholds,
                         int *int_distance_type, int *calc_ENTR, int *int_comp_platform) {
    Accrqa_Error error = SUCCESS;
    Accrqa_Distance dist = distance_of(int_distance_type[0], &error);
    if (error != SUCCESS) return;
    Accrqa_CompPlatform plt = platform_of(int_comp_platform[0], &error);
    if (error != SUCCESS) return;
    accrqa_LAM(output, input, (size_t)input_size[0], tau_values, nTaus[0], emb_values,
               nEmbs[0], vmin_values, nVmins[0], threshold_values, nThresholds[0], dist,
               calc_ENTR[0], plt, &error);
}

void R_double_accrqa_RR(double *output, double *input, int *input_size, int *tau_values,
                        int *nTaus, int *emb_values, int *nEmbs, double *threshold_values,
                        int *nThresholds, int *int_distance_type, int *int_comp_platform) {
    Accrqa_Error error = SUCCESS;
    Accrqa_Distance dist = distance_of(int_distance_type[0], &error);
    if (error != SUCCESS) return;
    Accrqa_CompPlatform plt = platform_of(int_comp_platform[0], &error);
    if (error != SUCCESS) return;
    accrqa_RR(output, input, (size_t)input_size[0], tau_values, nTaus[0], emb_values,
              nEmbs[0], threshold_values, nThresholds[0], dist, plt, &error);
}

void R_double_accrqa_RP(int *output, double *input, int *input_size, int *tau, int *emb,
                        double *threshold, int *int_distance_type) {
    Accrqa_Error error = SUCCESS;
    Accrqa_Distance dist = distance_of(int_distance_type[0], &error);
    if (error != SUCCESS) return;
    accrqa_RP(output, input, (size_t)input_size[0], tau[0], emb[0], threshold[0], dist,
              &error);
}

// src/AccRQA_threads.cpp:10-47.  The engine does its host work on the calling
// thread, so the count is recorded and reported but drives no thread pool.
static int g_threads = 0;

void accrqa_set_num_threads(int n) { g_threads = n < 1 ? 1 : n; }
int accrqa_get_max_threads(void) { return 1; }
int accrqa_get_num_threads(void) { return g_threads > 0 ? g_threads : 1; }

void R_accrqa_set_num_threads(int *n) {
    if (n) accrqa_set_num_threads(n[0]);
}
void R_accrqa_get_max_threads(int *out) {
    if (out) out[0] = accrqa_get_max_threads();
}
void R_accrqa_get_num_threads(int *out) {
    if (out) out[0] = accrqa_get_num_threads();
}

}  // extern "C"

#ifdef ACCRQA_R_FOUND
// Registration of the .C routines (src/AccRQA_R_bindings.cpp:250-262); built
// only where R's headers are available.
#include <R.h>
#include <R_ext/Rdynload.h>
extern "C" {
static R_CMethodDef accrqa_c_methods[] = {
    {"R_double_accrqa_DET", (DL_FUNC)&R_double_accrqa_DET, 14},
    {"R_double_accrqa_LAM", (DL_FUNC)&R_double_accrqa_LAM, 14},
    {"R_double_accrqa_RR", (DL_FUNC)&R_double_accrqa_RR, 11},
    {"R_double_accrqa_RP", (DL_FUNC)&R_double_accrqa_RP, 7},
    {"R_accrqa_set_num_threads", (DL_FUNC)&R_accrqa_set_num_threads, 1},
    {"R_accrqa_get_max_threads", (DL_FUNC)&R_accrqa_get_max_threads, 1},
    {"R_accrqa_get_num_threads", (DL_FUNC)&R_accrqa_get_num_threads, 1},
    {NULL, NULL, 0}};
void R_init_AccRQA(DllInfo *info) {
    R_registerRoutines(info, accrqa_c_methods, NULL, NULL, NULL);
    R_useDynamicSymbols(info, FALSE);
}
}
#endif
