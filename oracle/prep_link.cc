// ORACLE — test infrastructure only (the CPU port of the locarna pipeline,
// oracle/port_locarna.cc). Link stubs that let the host table preparation
// (locarna_gb300/csrc/host_prep.cpp) be compiled without the GPU engine: the
// error string of the C ABI, and the GPU envelope of lcg_prepare_pairs, which
// the port never calls (it uses lcg_prepare_pair, whose envelope is computed
// on the host in the reference's long double).
#include <string>

#include "../include/locarna_gb300.h"
#include "../locarna_gb300/csrc/envelope.hh"

static thread_local std::string g_err;

namespace lcg_host {
void set_error(const std::string &msg) { g_err = msg; }
}  // namespace lcg_host

extern "C" const char *lcg_last_error(void) { return g_err.c_str(); }

namespace lcg_env {
lcg_status compute(lcg_engine, const Params &, int, const PairIn *, PairOut *, std::string &err) {
    err = "the CPU port has no GPU envelope";
    return LCG_ERR_UNSUPPORTED;
}
lcg_status compute_begin(lcg_engine, const Params &, int, const PairIn *, PairOut *, Pending **pending,
                         std::string &err) {
    *pending = nullptr;
    err = "the CPU port has no GPU envelope";
    return LCG_ERR_UNSUPPORTED;
}
lcg_status compute_end(lcg_engine, Pending *, std::string &) { return LCG_OK; }
void reset_transfer(lcg_engine) {}
}  // namespace lcg_env
