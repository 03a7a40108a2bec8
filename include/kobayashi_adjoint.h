/*
 * kobayashi_adjoint.h -- reverse-mode gradients of a Kobayashi rollout.
 *
 * No counterpart in the reference (jklae/CrystalGrowth only runs the model
 * forward).  For the rollout of nsteps steps of src/Kobayashi.cpp:125-221
 * from an initial state (phi0, T0, theta0), with the loss
 *     L = 0.5 * sum over cells (phi_N - phi_target)^2,
 * kg_adjoint_gradient returns dL/d(delta, K, theta0, tau, gamma) and the
 * field dL/dT0.  The forward keeps a checkpoint of (phi, T, theta) every
 * `checkpoint_every` steps; the reverse sweep recomputes one segment at a
 * time, recording the per-cell intermediates on a tape, and runs the
 * hand-written adjoint of the fused step over it.  Gradients are reduced in
 * a fixed order, so repeated calls return identical bits.
 *
 * Branches of the model (the FLT_EPSILON dead zone of the angle, which keeps
 * theta; the constant +-pi/2 branches) are differentiated piecewise: inside
 * the dead zone the adjoint of theta passes straight to the previous step.
 */
#ifndef KOBAYASHI_ADJOINT_H
#define KOBAYASHI_ADJOINT_H
#include "kobayashi_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kg_grad_result {
    double loss;
    double d_delta, d_K, d_theta0, d_tau, d_gamma;
} kg_grad_result;

typedef struct kg_adjoint kg_adjoint;

/* nx x ny grid, nsteps >= 1 steps per rollout, checkpoint_every >= 1 */
KG_API int kg_adjoint_create(int nx, int ny, const kg_params* p, long long nsteps, int checkpoint_every,
                             kg_adjoint** out);
KG_API int kg_adjoint_destroy(kg_adjoint* a);
KG_API int kg_adjoint_set_params(kg_adjoint* a, const kg_params* p);
/* initial state (host buffers, nx*ny each; NULL theta = zeros) */
KG_API int kg_adjoint_set_initial(kg_adjoint* a, const double* phi0, const double* T0, const double* theta0);
/* phi_target (host buffer, nx*ny) */
KG_API int kg_adjoint_set_target(kg_adjoint* a, const double* phi_target);
/* forward rollout only: loss and the final state (any output may be NULL) */
KG_API int kg_adjoint_forward(kg_adjoint* a, double* loss, double* phi_N, double* T_N, double* theta_N);
/* forward rollout + reverse sweep; dL_dT0 (nx*ny) may be NULL */
KG_API int kg_adjoint_gradient(kg_adjoint* a, kg_grad_result* out, double* dL_dT0);
KG_API int kg_adjoint_get_stream(kg_adjoint* a, void** stream);

#ifdef __cplusplus
}
#endif
#endif
