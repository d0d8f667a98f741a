/* Learned absorbing edge for the GB300 time-stepping engine.
 *
 * No counterpart in the reference, which absorbs outgoing waves with a
 * TPML-cell PML on the left, right and bottom sides (ppml.F90).  Here a
 * thin PML (a few cells, the same PPML profiles) is followed, after every
 * time level, by a correction of the FDP_EDGE_DEPTH outermost cells of each
 * of those sides: for each such strip cell, a small network reads the 8
 * wavefield values (UM WM QX QZ TXX TZZ TXZ PRES) of the cell and of the
 * three cells inward of it, at the new level and at the two levels before,
 * and returns one additive correction per field.  There is one network per
 * side and depth (FDP_EDGE_SETS), each 96 -> 64 -> 64 -> 8 with tanh hidden
 * layers.  Inputs and outputs are divided by one scale per field.
 *
 * The networks are trained on the engine's own wavefields: a wide run with
 * the reference PML far away is the reflection-free target, and at every
 * level the thin-PML run restarts from the target's state (teacher
 * forcing), so each training sample asks for the correction that turns one
 * thin-PML level into the target's level.
 *
 * Arithmetic: weights and activations are rounded to bfloat16 and every
 * product is accumulated in FP32 -- tensor-core mma for the forward pass,
 * FP32 accumulation on the CUDA cores for the backward pass -- and the
 * optimizer (Adam) keeps FP32 master weights.  FP32 engines only.
 *
 * Parameters of one set, FP32, in this order: W1[64][96], b1[64],
 * W2[64][64], b2[64], W3[8][64], b3[8] (W[out][in]).
 */
#ifndef FDP_EDGE_H
#define FDP_EDGE_H

#include <stdint.h>

#include "fdp.h"

#ifdef __cplusplus
extern "C" {
#endif

#define FDP_EDGE_SIDES 3   /* 0 left, 1 right, 2 bottom */
#define FDP_EDGE_DEPTH 4   /* strip cells corrected per side */
#define FDP_EDGE_SETS 12   /* networks: side * FDP_EDGE_DEPTH + depth */
#define FDP_EDGE_IN 96     /* [level n, n-1, n-2][cell 0..3 inward][field] */
#define FDP_EDGE_HIDDEN 64
#define FDP_EDGE_OUT 8
#define FDP_EDGE_SET_PARAMS 10888

typedef struct fdp_edge fdp_edge;

/* Networks on `device` with weights drawn from a seeded uniform
 * distribution (+-1/sqrt(fan-in)), zero biases and zero output layer, so a
 * new edge corrects nothing; scale8 = per-field scales (NULL: all 1). */
int fdp_edge_create(int32_t device, const float* scale8, uint64_t seed, fdp_edge** out);

/* What the networks' outputs y do to a strip value v on the wavefield:
 * FDP_EDGE_CORRECT (the default) adds y * scale; FDP_EDGE_DAMP multiplies
 * v by 1 - sigmoid(y - 4), a per-field damping that can only remove
 * energy.  Training fits either kind to the same target values.  The
 * host-array entry points below always return the networks' raw outputs
 * and the loss of raw outputs against raw targets. */
#define FDP_EDGE_CORRECT 0
#define FDP_EDGE_DAMP 1
int fdp_edge_set_output(fdp_edge* e, int32_t kind);

/* All FDP_EDGE_SETS * FDP_EDGE_SET_PARAMS parameters, and the scales. */
int fdp_edge_get_params(fdp_edge* e, float* params);
int fdp_edge_set_params(fdp_edge* e, const float* params);
int fdp_edge_get_scale(fdp_edge* e, float* scale8);
int fdp_edge_set_scale(fdp_edge* e, const float* scale8);

/* The networks on host arrays: n samples, set[n] in 0..FDP_EDGE_SETS-1,
 * x[n][FDP_EDGE_IN] (already scaled), y[n][FDP_EDGE_OUT]. */
int fdp_edge_forward(fdp_edge* e, int32_t n, const int32_t* set, const float* x, float* y);

/* Loss = mean over samples and outputs of (y - target)^2; its gradient with
 * respect to all parameters (same layout as the parameters) and its value.
 * No update. */
int fdp_edge_gradients(fdp_edge* e, int32_t n, const int32_t* set, const float* x, const float* target,
                       float* grad, double* loss);

/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) with learning rate lr on
 * the loss of the given samples; *loss (may be NULL) receives its value
 * before the step. */
int fdp_edge_train_batch(fdp_edge* e, int32_t n, const int32_t* set, const float* x, const float* target, float lr,
                         double* loss);

/* One training level.  `trunc` (thin PML, MX x MZ) has just run level
 * `level`; `ext` (the wide target, whose cell (I + ox, L) is trunc's cell
 * (I, L)) has run the same level.  Gathers every strip cell's inputs and
 * target correction (ext's value minus trunc's), and takes one Adam step.
 * Then, with `teacher` set, copies ext's wavefield over trunc's grid and
 * records it as the history the next level's inputs use (teacher forcing:
 * trunc's next level starts from the target); without, applies the
 * correction the network gave before the step and records the corrected
 * values, exactly as an attached edge does (trunc runs on its own).  Both
 * contexts must be FP32 with the same free-surface mode, and ext's
 * interior (columns 1..MX, rows up to MZ) must hold trunc's whole grid
 * shifted by ox columns. */
int fdp_edge_train_level(fdp_edge* e, fdp_ctx* trunc, fdp_ctx* ext, int32_t ox, int32_t level, float lr,
                         int32_t teacher, double* loss);

/* Applies the edge after every level that fdp_run advances `trunc` by (NULL
 * detaches).  The edge must outlive the attachment.  Starts the input
 * history at rest; attach before level 1. */
int fdp_edge_attach(fdp_ctx* trunc, fdp_edge* e);

const char* fdp_edge_last_error(const fdp_edge* e);
void fdp_edge_destroy(fdp_edge* e);

#ifdef __cplusplus
}
#endif

#endif /* FDP_EDGE_H */
