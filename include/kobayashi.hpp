/*
 * kobayashi.hpp -- header-only C++ class over the C ABI (kobayashi_gpu.h)
 * with the simulation surface of the reference's class Kobayashi
 * (jklae/CrystalGrowth src/Kobayashi.h:32-122), headless.
 *
 * A caller of the reference replaces
 *     Kobayashi* sim = new Kobayashi(250, 250, 0.0001f);      // src/main.cpp:18
 *     sim->iUpdate();                                           // per frame
 * by the same lines with this header; the state then lives in HBM and phi()
 * copies it back for display.  The Win32/Direct3D methods of ISimulation
 * (src/Kobayashi.h:44-66) belong to the viewer and are not part of the
 * library; iGetObjectCount and iIsUpdated are kept.
 *
 * Errors from the C ABI become kg::Error exceptions here (the reference had
 * no error reporting at all).
 */
#pragma once
#include <stdexcept>
#include <string>
#include <vector>

#include "kobayashi_gpu.h"

namespace kg {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc)
{
    if (rc != KG_OK)
        throw Error(rc, kg_last_error());
}

struct Int3 {
    int x, y, z;
};

class Kobayashi {
  public:
    /* Kobayashi(int x, int y, float timeStep): src/Kobayashi.cpp:7-67 */
    Kobayashi(int x, int y, double timeStep)
    {
        kg_params p;
        check(kg_params_default(&p, timeStep));
        check(kg_create(x, y, &p, &h_));
    }
    Kobayashi(int x, int y, const kg_params& p) { check(kg_create(x, y, &p, &h_)); }
    ~Kobayashi() { kg_destroy(h_); }
    Kobayashi(const Kobayashi&) = delete;
    Kobayashi& operator=(const Kobayashi&) = delete;

    /* iUpdate: 10 explicit steps (src/Kobayashi.cpp:227-239) */
    void iUpdate() { check(kg_update(h_)); }
    /* iResetSimulationState: fields re-zeroed, nucleus re-seeded (src/Kobayashi.cpp:241-249) */
    void iResetSimulationState() { check(kg_reset(h_)); }
    /* iGetObjectCount (src/Kobayashi.cpp:363-366) */
    Int3 iGetObjectCount() const
    {
        int nx = 0, ny = 0;
        check(kg_get_size(h_, &nx, &ny));
        return {nx, ny, 0};
    }
    /* iIsUpdated (src/Kobayashi.cpp:378-381): the headless library always steps */
    bool iIsUpdated() const { return true; }

    /* extensions */
    void step(long long n) { check(kg_step(h_, n)); }
    void sync() { check(kg_sync(h_)); }
    kg_params params() const
    {
        kg_params p;
        check(kg_get_params(h_, &p));
        return p;
    }
    void setParams(const kg_params& p) { check(kg_set_params(h_, &p)); }
    void seedDisks(const std::vector<int>& cx, const std::vector<int>& cy, const std::vector<int>& r)
    {
        if (cx.size() != cy.size() || cx.size() != r.size())
            throw Error(KG_ERR_INVALID, "seedDisks: size mismatch");
        check(kg_seed_disks(h_, (int)cx.size(), cx.data(), cy.data(), r.data()));
    }
    std::vector<double> phi() const { return field(0); }
    std::vector<double> T() const { return field(1); }
    std::vector<double> theta() const { return field(2); }
    void setFields(const std::vector<double>& phi, const std::vector<double>& t, const std::vector<double>& th)
    {
        size_t n = cells();
        if (phi.size() != n || t.size() != n || th.size() != n)
            throw Error(KG_ERR_INVALID, "setFields: size mismatch");
        check(kg_set_fields(h_, phi.data(), t.data(), th.data()));
    }
    /* strip shape and temporal blocking (kg_set_tile, kg_set_tblock): speed only, the same bits */
    void setTile(int nt, int bh) { check(kg_set_tile(h_, nt, bh)); }
    void setTblock(int k) { check(kg_set_tblock(h_, k)); }
    int tblock() const
    {
        int k = 1;
        check(kg_get_tblock(h_, &k));
        return k;
    }
    long long steps() const
    {
        long long s = 0, f = 0;
        check(kg_get_counters(h_, &s, &f));
        return s;
    }
    long long frames() const
    {
        long long s = 0, f = 0;
        check(kg_get_counters(h_, &s, &f));
        return f;
    }
    kg_sim* handle() const { return h_; }

  private:
    size_t cells() const
    {
        Int3 c = iGetObjectCount();
        return (size_t)c.x * (size_t)c.y;
    }
    std::vector<double> field(int which) const
    {
        std::vector<double> out(cells());
        double* p[3] = {nullptr, nullptr, nullptr};
        p[which] = out.data();
        check(kg_get_fields(h_, p[0], p[1], p[2]));
        return out;
    }
    kg_sim* h_ = nullptr;
};

} // namespace kg
