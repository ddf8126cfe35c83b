/*****************************************************************************
 *
 *  abi_probe.c  (test program)
 *
 *  Prints, as one JSON object, the size and member offsets of every
 *  structure a caller of the drop-in interface fills or reads, and the
 *  values of its enumerations.  Compiled once against include/ludwig_gb.h
 *  and once against the reference's own headers (-DPROBE_REFERENCE, with
 *  the reference's src/, target/ and mpi_s/ on the include path), the two
 *  outputs must be identical: code compiled against either header agrees
 *  on every offset.
 *
 *****************************************************************************/

#include <stddef.h>
#include <stdio.h>

#ifdef PROBE_REFERENCE
#include "free_energy.h"
#include "lb_data_options.h"
#include "field_options.h"
#include "hydro_options.h"
#include "map.h"
#include "symmetric.h"
#include "blue_phase.h"
#include "blue_phase_beris_edwards.h"
#include "phi_cahn_hilliard.h"
#include "memory.h"
#else
#include "ludwig_gb.h"
#endif

static int first = 1;

static void kv(const char * key, long v) {
  printf("%s\"%s\": %ld", first ? "{" : ", ", key, v);
  first = 0;
}

#define SZ(T) kv("sizeof(" #T ")", (long) sizeof(T))
#define OFF(T, m) kv("offsetof(" #T "," #m ")", (long) offsetof(T, m))
#define VAL(e) kv(#e, (long) (e))

int main(void) {

  SZ(struct fe_s);
  OFF(struct fe_s, func);
  OFF(struct fe_s, id);
  OFF(struct fe_s, use_stress_relaxation);

  SZ(fe_vt_t);
  OFF(fe_vt_t, free);
  OFF(fe_vt_t, target);
  OFF(fe_vt_t, fed);
  OFF(fe_vt_t, mu);
  OFF(fe_vt_t, mu_solv);
  OFF(fe_vt_t, stress);
  OFF(fe_vt_t, str_symm);
  OFF(fe_vt_t, str_anti);
  OFF(fe_vt_t, hvector);
  OFF(fe_vt_t, htensor);
  OFF(fe_vt_t, htensor_v);
  OFF(fe_vt_t, stress_v);
  OFF(fe_vt_t, str_symm_v);
  OFF(fe_vt_t, str_anti_v);

  VAL(FE_NULL); VAL(FE_SYMMETRIC); VAL(FE_BRAZOVSKII); VAL(FE_SURFACTANT);
  VAL(FE_POLAR); VAL(FE_LC); VAL(FE_ELECTRO); VAL(FE_ELECTRO_SYMMETRIC);
  VAL(FE_LC_DROPLET); VAL(FE_TERNARY);
  VAL(NSIMDVL);

  SZ(io_options_t);
  OFF(io_options_t, mode);
  OFF(io_options_t, iorformat);
  OFF(io_options_t, metadata_version);
  OFF(io_options_t, report);
  OFF(io_options_t, asynchronous);
  OFF(io_options_t, compression_levl);
  OFF(io_options_t, iogrid);
  SZ(io_info_args_t);
  OFF(io_info_args_t, input);
  OFF(io_info_args_t, output);
  OFF(io_info_args_t, grid);
  OFF(io_info_args_t, iofreq);
  VAL(IO_MODE_MPIIO); VAL(IO_RECORD_ASCII); VAL(IO_RECORD_BINARY);
  VAL(IO_METADATA_SINGLE_V1); VAL(IO_METADATA_V2);

  SZ(lb_data_options_t);
  OFF(lb_data_options_t, ndim);
  OFF(lb_data_options_t, nvel);
  OFF(lb_data_options_t, ndist);
  OFF(lb_data_options_t, nrelax);
  OFF(lb_data_options_t, halo);
  OFF(lb_data_options_t, reportimbalance);
  OFF(lb_data_options_t, usefirsttouch);
  OFF(lb_data_options_t, iodata);
  VAL(LB_RELAXATION_M10); VAL(LB_RELAXATION_BGK); VAL(LB_RELAXATION_TRT);
  VAL(LB_HALO_FULL); VAL(LB_HALO_REDUCED);

  SZ(field_options_t);
  OFF(field_options_t, ndata);
  OFF(field_options_t, nhcomm);
  OFF(field_options_t, haloscheme);
  OFF(field_options_t, haloverbose);
  OFF(field_options_t, usefirsttouch);
  OFF(field_options_t, iodata);
  VAL(FIELD_HALO_HOST); VAL(FIELD_HALO_TARGET); VAL(FIELD_HALO_OPENMP);

  SZ(hydro_options_t);
  OFF(hydro_options_t, nhcomm);
  OFF(hydro_options_t, rho);
  OFF(hydro_options_t, u);
  OFF(hydro_options_t, force);
  OFF(hydro_options_t, eta);

  SZ(map_options_t);
  OFF(map_options_t, ndata);
  OFF(map_options_t, is_porous_media);
  OFF(map_options_t, filestub);
  OFF(map_options_t, iodata);
  VAL(MAP_FLUID); VAL(MAP_BOUNDARY); VAL(MAP_COLLOID); VAL(MAP_STATUS_MAX);

  SZ(fe_symm_param_t);
  OFF(fe_symm_param_t, a);
  OFF(fe_symm_param_t, b);
  OFF(fe_symm_param_t, kappa);
  OFF(fe_symm_param_t, c);
  OFF(fe_symm_param_t, h);

  SZ(lc_anchoring_param_t);
  OFF(lc_anchoring_param_t, type);
  OFF(lc_anchoring_param_t, w1);
  OFF(lc_anchoring_param_t, w2);
  OFF(lc_anchoring_param_t, nfix);
  VAL(LC_ANCHORING_NONE); VAL(LC_ANCHORING_PLANAR); VAL(LC_ANCHORING_NORMAL);
  VAL(LC_ANCHORING_FIXED); VAL(LC_ANCHORING_INVALID);

  SZ(fe_lc_param_t);
  OFF(fe_lc_param_t, a0);
  OFF(fe_lc_param_t, q0);
  OFF(fe_lc_param_t, gamma);
  OFF(fe_lc_param_t, kappa0);
  OFF(fe_lc_param_t, kappa1);
  OFF(fe_lc_param_t, xi);
  OFF(fe_lc_param_t, zeta0);
  OFF(fe_lc_param_t, zeta1);
  OFF(fe_lc_param_t, zeta2);
  OFF(fe_lc_param_t, redshift);
  OFF(fe_lc_param_t, rredshift);
  OFF(fe_lc_param_t, epsilon);
  OFF(fe_lc_param_t, amplitude0);
  OFF(fe_lc_param_t, e0);
  OFF(fe_lc_param_t, coswt);
  OFF(fe_lc_param_t, is_redshift_updated);
  OFF(fe_lc_param_t, is_active);
  OFF(fe_lc_param_t, coll);
  OFF(fe_lc_param_t, wall);

  SZ(beris_edw_param_t);
  OFF(beris_edw_param_t, xi);
  OFF(beris_edw_param_t, gamma);
  OFF(beris_edw_param_t, noise);
  OFF(beris_edw_param_t, var);
  OFF(beris_edw_param_t, tmatrix);

  SZ(phi_ch_info_t);
  OFF(phi_ch_info_t, conserve);
  OFF(phi_ch_info_t, noise);

  printf("}\n");
  return 0;
}
