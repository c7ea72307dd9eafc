// Stand-in of the C ABI (include/sdm_capi.h) for CPU tests of the force
// plugin's host logic: the entry points the plugin calls, with results that
// follow from the parameters alone (no force evaluation).
//   results[SDM_R_EPOT]       = 100 lambda
//   results[SDM_R_DWDLAMBDA]  = 3 + 2 lambda
//   results[SDM_R_RESERVED]   = number of sdm_set_params calls on this handle
//   results[SDM_R_U0]         = the handle's box edge x
//   results[SDM_R_U1]         = number of sdm_create calls in the process
//   results[SDM_R_U], [SDM_R_W], [SDM_R_DW] = 7, 11, 13
// Forces are zero.
#include "sdm_capi.h"

#include <cstring>
#include <new>

static int g_creates = 0;

struct sdm_handle {
    int n = 0;
    double box0 = 0.0;
    int set_params_calls = 0;
    double p[SDM_NPARAMS] = {};
};

extern "C" {

sdm_status sdm_create(const sdm_system_desc* systems, int num_systems, int, sdm_handle** out) {
    if (!out || !systems || num_systems != 1) return SDM_ERR_INVALID_ARGUMENT;
    sdm_handle* h = new (std::nothrow) sdm_handle();
    if (!h) return SDM_ERR_INVALID_ARGUMENT;
    h->n = systems[0].num_particles;
    h->box0 = systems[0].box[0];
    ++g_creates;
    *out = h;
    return SDM_OK;
}

sdm_status sdm_destroy(sdm_handle* h) {
    delete h;
    return SDM_OK;
}

const char* sdm_last_error(const sdm_handle*) { return "fake"; }

sdm_status sdm_set_params(sdm_handle* h, int replica, const double* params) {
    if (!h || replica != 0 || !params) return SDM_ERR_INVALID_ARGUMENT;
    std::memcpy(h->p, params, sizeof(h->p));
    h->set_params_calls++;
    return SDM_OK;
}

// refuses displacement components beyond 1e6 nm (a library-side refusal
// for the plugin's all-or-nothing update test)
sdm_status sdm_set_displacement(sdm_handle* h, int system, const double* d) {
    if (!h || system != 0 || !d) return SDM_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < 3 * h->n; ++k)
        if (d[k] > 1.0e6) return SDM_ERR_INVALID_ARGUMENT;
    return SDM_OK;
}

sdm_status sdm_evaluate(sdm_handle* h, const double* x, double* results, double* forces) {
    if (!h || !x) return SDM_ERR_INVALID_ARGUMENT;
    const double lam = h->p[SDM_P_LAMBDA];
    if (results) {
        for (int k = 0; k < SDM_NRESULTS; ++k) results[k] = 0.0;
        results[SDM_R_EPOT] = 100.0 * lam;
        results[SDM_R_DWDLAMBDA] = 3.0 + 2.0 * lam;
        results[SDM_R_RESERVED] = h->set_params_calls;
        results[SDM_R_U0] = h->box0;
        results[SDM_R_U1] = g_creates;
        results[SDM_R_U] = 7.0;
        results[SDM_R_W] = 11.0;
        results[SDM_R_DW] = 13.0;
    }
    if (forces) std::memset(forces, 0, 3 * (size_t)h->n * sizeof(double));
    return SDM_OK;
}

}  // extern "C"
