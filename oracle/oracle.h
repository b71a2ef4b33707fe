/*
 * oracle.h -- CPU restatement of BookLeaf's per-step hydro path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GB300 path is compared
 * against; it is never linked into, loaded by or called from the product
 * library.  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline
 * leg may use it.
 *
 * PARITY STATUS: the reference (Fortran 2008) cannot be compiled where this
 * project is built (no Fortran compiler), and it ships no golden vectors.
 * The restatement is therefore pinned only by the reference's own known-
 * answer test, the Sod shock-tube L1 density norm against the exact Riemann
 * solution (src/packages/check/kernel/check_kn_tests.f90:33-111), and by
 * conservation invariants.  Bitwise parity with the reference serial build
 * is "parity unpinned".
 *
 * The entry points operate in place on the caller's host arrays, registered
 * by dataAPI ID exactly like bl_init (include/bookleaf_gb300.h), and follow
 * the reference's routines statement by statement, including its scratch
 * aliasing (src/dataAPI/dataAPI_id.f90:78-111).  Build with
 * -ffp-contract=off so that no multiply-add is fused.
 */
#ifndef BOOKLEAF_ORACLE_H
#define BOOKLEAF_ORACLE_H

#include "../include/bookleaf_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

orc_ctx *orc_init(const bl_sizes *sizes, const bl_config *config,
                  void *const *dh, bl_error *error);
void orc_finalize(orc_ctx *ctx);

/* inf_solver_getdt / inf_solver_lagstep / inf_solver_alestep */
int orc_getdt(orc_ctx *ctx, bl_timestep *ts, bl_error *error);
int orc_lagstep(orc_ctx *ctx, bl_timestep *ts, bl_error *error);
int orc_alestep(orc_ctx *ctx, const bl_timestep *ts, bl_error *error);

/* Host pointer of field id (scratch fields are allocated by the oracle when
 * the caller registered none). */
void *orc_field(orc_ctx *ctx, int id);

/* check_kn_sod (check_kn_tests.f90:33-62) + check_dr_sod normalisation
 * (check_dr_tests.f90:34-71): volume-weighted L1 norms of density and energy
 * against the exact Sod solution, geometry x in [0,100], interface at 50. */
void orc_sod_l1(int nel, double time, const double *volume,
                const double *density, const double *energy,
                const double *cnx, const double *cny, double out[2]);

/* geometry_kn_getcentroid (geometry_kn_centroid.f90:29-55) */
void orc_centroid(int nvert, const double *xx, const double *yy, double c[2]);

/* exp, log and ** of the equations of state (eos_kn_forms.f90), evaluated
 * with the same operations as the device's (see oracle.c) */
double orc_exp(double x);
double orc_log(double a);
double orc_pow(double a, double b);

#ifdef __cplusplus
}
#endif

#endif
