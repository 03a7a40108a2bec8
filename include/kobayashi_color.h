/*
 * kobayashi_color.h -- the reference's phi -> RGBA colour ramp, headless.
 *
 * Replaces Kobayashi::iUpdateConstantBuffer (src/Kobayashi.cpp:309-345),
 * which the DXViewer loop calls once per cell per frame to fill Direct3D
 * constant buffers: one call here colours every cell of a kg_sim's current phi
 * (RGBA float32, alpha 1), with the reference's FP64-build arithmetic.
 */
#ifndef KOBAYASHI_COLOR_H
#define KOBAYASHI_COLOR_H
#include "kobayashi_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define KG_COLOR_GRID 0   /* rgba[4 (i + nx j) + c]: colour of cell (i, j) */
#define KG_COLOR_VIEWER 1 /* the viewer's constant-buffer order, with the reference's transposition
                             (cell i coloured from phi at (i / s, i % s), s = sqrt(nx ny)); square grids */

/* 4 nx ny floats into a host buffer (synchronous) */
KG_API int kg_colormap(kg_sim* h, int order, float* rgba);
/* the same into a 16-byte aligned device buffer, enqueued on the handle's stream */
KG_API int kg_colormap_device(kg_sim* h, int order, float* rgba_device);

#ifdef __cplusplus
}
#endif
#endif
