// Drives include/kobayashi.hpp the way src/main.cpp drives the reference's class:
// construct with (x, y, timeStep), call iUpdate() per frame, read phi.  Prints
// the step/frame counters and a checksum of the fields so the test can compare
// them with the same run through the Python binding.
#include <cstdio>
#include <cstring>
#include <cstdint>
#include "kobayashi.hpp"

static uint64_t fnv(const std::vector<double>& v, uint64_t h)
{
    const unsigned char* p = reinterpret_cast<const unsigned char*>(v.data());
    for (size_t i = 0; i < v.size() * sizeof(double); i++) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

int main()
{
    try {
        kg::Kobayashi sim(250, 250, 0.0001);  // src/main.cpp:14-18
        for (int frame = 0; frame < 30; frame++)
            sim.iUpdate();
        kg::Int3 n = sim.iGetObjectCount();
        uint64_t h = 1469598103934665603ull;
        h = fnv(sim.phi(), h);
        h = fnv(sim.T(), h);
        h = fnv(sim.theta(), h);
        std::printf("%d %d %lld %lld %016llx\n", n.x, n.y, sim.steps(), sim.frames(), (unsigned long long)h);
        sim.iResetSimulationState();
        std::printf("reset %lld %lld\n", sim.steps(), sim.frames());
        bool caught = false;
        try {
            kg_params p = sim.params();
            p.tau = -1.0;
            sim.setParams(p);
        } catch (const kg::Error& e) {
            caught = e.code == KG_ERR_INVALID;
        }
        std::printf("invalid params rejected %d\n", caught ? 1 : 0);
        // the same 30 frames with two time steps per pass: the same bits
        kg::Kobayashi sim2(250, 250, 0.0001);
        sim2.setTblock(2);
        for (int frame = 0; frame < 30; frame++)
            sim2.iUpdate();
        uint64_t h2 = 1469598103934665603ull;
        h2 = fnv(sim2.phi(), h2);
        h2 = fnv(sim2.T(), h2);
        h2 = fnv(sim2.theta(), h2);
        std::printf("tblock %d same %d\n", sim2.tblock(), h2 == h ? 1 : 0);
    } catch (const kg::Error& e) {
        std::printf("error %d %s\n", e.code, e.what());
        return 1;
    }
    return 0;
}
