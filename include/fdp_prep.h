/*
 * fdp_prep.h -- host-side set-up that produces the inputs of fdp.h.
 *
 * In the reference these steps run once in the Fortran driver before
 * TIME_LOOP (main.F90:60-82); the drop-in keeps them on the host.  With no
 * Fortran compiler available they are restated in C++ here, with the
 * reference's arithmetic (precision PP chosen by `prec`, FDP_F32 or
 * FDP_F64).  All functions return FDP_OK or a negative FDP_ERR_* code.
 */
#ifndef FDP_PREP_H
#define FDP_PREP_H

#include <stdint.h>

#include "fdp.h"

#ifdef __cplusplus
extern "C" {
#endif

/* CALCUL_VELOCITY (calcul_velocity.F90:1-37): fast-P, slow-P and S speeds
 * of one material from SIG_1, P, AINV, MU and the unscaled REL1..3.
 * Values in/out are doubles holding numbers of precision `prec`. */
int fdp_prep_velocities(int32_t prec, double sig1, double p, double ainv, double mu, double rel1,
                        double rel2, double rel3, double* vpf, double* vps, double* vs);

/* READ_MODEL_PAR scaling (read_model_par.F90:63-74) of a .MO table
 * table24[(jm-1)*24+k] in place. */
int fdp_prep_scale_table(int32_t prec, int32_t jmnum, double dt, double h, void* table24);

/* READ_MODEL (read_model.F90:57-89): expands the physical JM rows read from
 * the .JMH file, jm_rows[r*mx + (i-1)], r = 0.. (rows 2..MZ under stress
 * imaging, 0..MZ without), into JM(PMLL:PMLXH, 0:PMLZH). */
int fdp_prep_expand_jm(int32_t mx, int32_t mz, int32_t tpml, int32_t stress_imaging, const int32_t* jm_rows,
                       int32_t* jm_out);

/* PPML (ppml.F90:156-306): the 24 damping profiles in fdp_set_pml order.
 * r, tau, pow, sf, wc are CONTROLDATA1 values (read_open.F90:54,118-126),
 * ktbo the bottom condition key. */
int fdp_prep_pml(int32_t prec, int32_t mx, int32_t mz, int32_t tpml, int32_t ktbo, double r, double tau,
                 double pow_, double sf, double wc, double dt, double h, const int32_t* jm, int32_t jmnum,
                 const void* table24, void* const* profiles24);

/* PRE_NR_COEF1 bottom part (pre_nr_coef1.F90:187-202) with NONREF
 * (nonref.F90:69-204), HIGDON_FD, HIGCE_FD, HIGCE2_FD and OptAbsBc:
 * the 16 coefficients ABW01..ABW22, ABH01..ABH22.  omg is the NONREF
 * namelist OMG already divided by 2*pi (read_open.F90:188). */
int fdp_prep_bottom_nr(int32_t prec, int32_t mx, int32_t mz, int32_t tpml, int32_t ktbo, double dt, double h,
                       double omg, double wb, double thpple, double thssle, const int32_t* jm, int32_t jmnum,
                       const void* table24, void* ab16);

/* OPEN_SR_FILE (open_sr_file.F90:41-110): cubic-spline resampling of the
 * STF.DAT samples (time[k], stf[k], k < nstf) to the levels 1..MT2 with the
 * reference's clamped end conditions, zero after the last sample, split
 * into solid/fluid parts by key_sour and qr, and divided by H**2.
 * Output SOURTF_A(2, MT2) column-major. */
int fdp_prep_source(int32_t prec, int32_t nstf, const void* time, const void* stf, int32_t mt2, double dt,
                    double h, int32_t key_sour, double qr, void* sourtf);

#ifdef __cplusplus
}
#endif

#endif /* FDP_PREP_H */
