/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE ONLY (the "O1" oracle).
 *
 * Wraps the reference's own, unmodified src/Kobayashi.cpp (jklae/CrystalGrowth)
 * in a small C API so tests and the CPU baseline can drive it through ctypes.
 * build_oracle.py compiles it twice against the Linux shim in ref_shim/:
 *   -DKO_REF_FP64 : "#define float double" before the include, i.e. the
 *                   reference's algorithm verbatim in FP64 (symbols ref64_*)
 *   (default)     : the reference as shipped, FP32 (symbols ref32_*)
 * "#define private public" exposes the fields (src/Kobayashi.h:80-121).
 * Never linked into the product.
 */
#include <vector>
#include <string>
#include <cmath>
#include <cfloat>
#include <ctime>
#include <cstdio>
#include <cstring>

#define private public
#ifdef KO_REF_FP64
#define float double
#endif
#include "Kobayashi.cpp"
#ifdef KO_REF_FP64
#undef float
#endif
#undef private

#ifdef KO_REF_FP64
typedef double ref_real;
#define REF(name) ref64_##name
#else
typedef float ref_real;
#define REF(name) ref32_##name
#endif

#pragma GCC visibility push(default)
extern "C" {

/* Kobayashi(int x, int y, float timeStep): src/Kobayashi.cpp:7-67 */
void* REF(create)(int nx, int ny, double dt)
{
    return new Kobayashi(nx, ny, (ref_real)dt);
}

void REF(destroy)(void* h) { delete (Kobayashi*)h; }

/* p: dx, dy, dt, tau, eps_bar, mu, K, delta, aniso, alpha, gamma, teq
 * (overwrites the float literals assigned at src/Kobayashi.cpp:61-63,76-84) */
void REF(set_params)(void* h, const double* p)
{
    Kobayashi* k = (Kobayashi*)h;
    k->_dx = (ref_real)p[0];
    k->_dy = (ref_real)p[1];
    k->_dt = (ref_real)p[2];
    k->_tau = (ref_real)p[3];
    k->_epsilonBar = (ref_real)p[4];
    k->_mu = (ref_real)p[5];
    k->_K = (ref_real)p[6];
    k->_delta = (ref_real)p[7];
    k->_anisotropy = (ref_real)p[8];
    k->_alpha = (ref_real)p[9];
    k->_gamma = (ref_real)p[10];
    k->_tEq = (ref_real)p[11];
}

void REF(get_params)(void* h, double* p)
{
    Kobayashi* k = (Kobayashi*)h;
    p[0] = k->_dx; p[1] = k->_dy; p[2] = k->_dt; p[3] = k->_tau; p[4] = k->_epsilonBar; p[5] = k->_mu;
    p[6] = k->_K; p[7] = k->_delta; p[8] = k->_anisotropy; p[9] = k->_alpha; p[10] = k->_gamma; p[11] = k->_tEq;
}

void REF(set_state)(void* h, const double* phi, const double* t, const double* theta)
{
    Kobayashi* k = (Kobayashi*)h;
    for (size_t i = 0; i < k->_phi.size(); i++) {
        k->_phi[i] = (ref_real)phi[i];
        k->_t[i] = (ref_real)t[i];
        k->_angl[i] = (ref_real)theta[i];
    }
}

void REF(get_state)(void* h, double* phi, double* t, double* theta)
{
    Kobayashi* k = (Kobayashi*)h;
    for (size_t i = 0; i < k->_phi.size(); i++) {
        phi[i] = k->_phi[i];
        t[i] = k->_t[i];
        theta[i] = k->_angl[i];
    }
}

/* one explicit step = _computeGradientLaplacian + _evolution (src/Kobayashi.cpp:232-233) */
void REF(step)(void* h, long long n)
{
    Kobayashi* k = (Kobayashi*)h;
    for (long long s = 0; s < n; s++) {
        k->_computeGradientLaplacian();
        k->_evolution();
    }
}

/* iUpdate: 10 steps per call (src/Kobayashi.cpp:227-239) */
void REF(update)(void* h) { ((Kobayashi*)h)->iUpdate(); }

/* _vectorInit: zero fields + 5-cell nucleus (src/Kobayashi.cpp:98-123) */
void REF(vector_init)(void* h) { ((Kobayashi*)h)->_vectorInit(); }

int REF(frame)(void* h) { return ((Kobayashi*)h)->_simFrame; }

/* colours of all cells of a square grid, in the viewer's cell order
 * (src/Kobayashi.cpp:309-345 called for i = 0..N-1); rgba: 4*N floats */
void REF(colors)(void* h, float* rgba)
{
    Kobayashi* k = (Kobayashi*)h;
    std::vector<ConstantBuffer> cb((size_t)k->_objectCount.x * k->_objectCount.y);
    for (int i = 0; i < (int)cb.size(); i++) {
        k->iUpdateConstantBuffer(cb, i);
        rgba[4 * i + 0] = (float)cb[i].color.x;
        rgba[4 * i + 1] = (float)cb[i].color.y;
        rgba[4 * i + 2] = (float)cb[i].color.z;
        rgba[4 * i + 3] = (float)cb[i].color.w;
    }
}

} /* extern "C" */
#pragma GCC visibility pop
