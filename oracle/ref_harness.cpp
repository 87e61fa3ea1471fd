// ref_harness.cpp -- C entry points around the reference's own pricer, compiled
// together with the reference sources into oracle/_ref/libkwref.so by
// oracle/Makefile.  TEST INFRASTRUCTURE ONLY: used to pin the oracle
// restatement (fd1d_oracle.c) and to generate the golden fixtures; nothing in the
// product links it.
//
// It drives the reference exactly as its tests do (test/kwPricer_test.cpp:63-84):
// a kw::Config with PRICER and the FD1D.* keys (src/Pricer/kwFd1d.cpp:9-19), then
// kw::PricerFactory::create and Pricer::price (src/Pricer/kwPricerFactory.h:15-41).
#include <chrono>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "Core/kwAsset.h"
#include "Core/kwConfig.h"
#include "Pricer/kwPricerFactory.h"
#include "kwThreadPool.h"

struct kwref_option {  // same layout as kw::Option
    double t, k, z, r, q, s;
    uint8_t e;
    int8_t w;
};
static_assert(sizeof(kwref_option) == sizeof(kw::Option), "layout");

extern "C" {

// Returns 0 on success; otherwise 1 and the reference's error string in err.
// Negative density / scale / dims mean "leave the key unset" (reference default).
int kwref_price(const char* pricer, const kwref_option* opts, size_t n, double density,
                double scale, long t_dim, long x_dim, double* prices, char* err, size_t errlen,
                double* seconds)
{
    std::vector<kw::Option> assets(n);
    for (size_t i = 0; i < n; ++i) {
        kw::Option& a = assets[i];
        a.t = opts[i].t;
        a.k = opts[i].k;
        a.z = opts[i].z;
        a.r = opts[i].r;
        a.q = opts[i].q;
        a.s = opts[i].s;
        a.e = opts[i].e;
        a.w = opts[i].w;
    }
    kw::Config config;
    config.set("PRICER", std::string(pricer));
    if (density > 0) config.set("FD1D.DENSITY", density);
    if (scale > 0) config.set("FD1D.SCALE", scale);
    if (t_dim > 0) config.set("FD1D.T_GRID_SIZE", (int64_t)t_dim);
    if (x_dim > 0) config.set("FD1D.X_GRID_SIZE", (int64_t)x_dim);

    kw::sPtr<kw::Pricer> p;
    std::string e = kw::PricerFactory::create(config, p);
    if (!e.empty()) {
        if (err) snprintf(err, errlen, "%s", e.c_str());
        return 1;
    }
    std::vector<double> out;
    auto t0 = std::chrono::steady_clock::now();
    e = p->price(assets, out);
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    for (size_t i = 0; i < n && i < out.size(); ++i) prices[i] = out[i];
    if (!e.empty()) {
        if (err) snprintf(err, errlen, "%s", e.c_str());
        return 1;
    }
    return 0;
}

// Threads the reference's pool runs (std::thread::hardware_concurrency()).
int kwref_pool_size() { return (int)kw::ThreadPool::instance().size(); }

}  // extern "C"
