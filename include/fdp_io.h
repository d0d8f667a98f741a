/*
 * fdp_io.h -- the reference's file formats, for hosts without the Fortran
 * driver (the C++ drop-in host fdp_host uses them).
 *
 *   - Fortran namelist input (<JOB>.IN, <JOB>.INM; read_open.F90:48-69)
 *   - gfortran unformatted sequential records with 4-byte length markers
 *     (.JMH and .MO, read_model.F90:62, read_model_par.F90:37-60;
 *     SNAP.V######, store_snapshots.F90:173-190)
 *   - the Ew.d edit descriptor of the seismogram files
 *     ('(5(1X,E13.6))', store_seismograms.F90:144)
 *
 * All functions return FDP_OK or a negative FDP_ERR_* code.
 */
#ifndef FDP_IO_H
#define FDP_IO_H

#include <stddef.h>
#include <stdint.h>

#include "fdp.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Formats `value` with the Fortran edit descriptor Ew.d as gfortran writes
 * it (e.g. E13.6: " 0.123457E+01"); out must hold w+1 bytes.  A value that
 * does not fit is written as w asterisks, as Fortran does. */
int fdp_io_format_e(double value, int32_t w, int32_t d, char* out);

/* Parses the namelist group `group` (case-insensitive) from the text `text`
 * and looks up `name`: copies the value's text (quotes removed) into out
 * (size bytes).  Returns FDP_OK, or FDP_ERR_ARG when the group or the name
 * is absent. */
int fdp_io_namelist_get(const char* text, const char* group, const char* name, char* out, size_t size);

/* Reads record `index` (0-based) of a gfortran unformatted sequential file
 * into buf (capacity bytes); *nbytes receives the record length.  Records
 * longer than 2 GiB, written by gfortran as subrecords, are joined. */
int fdp_io_read_record(const char* path, int64_t index, void* buf, int64_t capacity, int64_t* nbytes);

/* Appends one record of nbytes bytes to a gfortran unformatted sequential
 * file (created when absent). */
int fdp_io_append_record(const char* path, const void* buf, int64_t nbytes);

#ifdef __cplusplus
}
#endif

#endif /* FDP_IO_H */
