/* Internal helpers shared by the oracle translation units (test only). */
#ifndef EMC_ORACLE_INTERNAL_H
#define EMC_ORACLE_INTERNAL_H
#include "emc_oracle.h"

/* per particle-step draw context */
typedef struct {
  oc_rng *r;
  int32_t mode;
  uint32_t ctr[4];
  uint32_t key[2];
  uint64_t buf[2];
  int32_t nbuf;
  int32_t fail; /* replay log exhausted */
} dctx;


void oci_dctx_init(dctx *d, oc_rng *r, uint32_t pid, uint32_t step, uint32_t streamWord);
uint64_t oci_draw_u64(dctx *d);
double oci_draw_u01(dctx *d);
double oci_draw_ulog(dctx *d);
void oci_grain_scatter(const oc_model *m, double *k, dctx *d);
double oci_grain_tau(const oc_model *m);
int32_t oci_surface(const oc_model *m, int32_t boundary, double *param);
uint32_t oci_draw_pick(dctx *d, uint32_t n);
int32_t oci_handler_scatter(const oc_model *m, double *k, double *E, int32_t *valley,
                            int32_t *sub, int32_t region, dctx *d);
double oci_new_tau(const oc_model *m, int32_t valley, int32_t region, dctx *d);
void oci_init_pos(const int64_t *coord, const int64_t *ext, const double *h, int32_t dim,
                  dctx *d, double *pos);
void oci_init_particle(const oc_model *m, const int64_t *coord, const int64_t *ext,
                       const double *h, int32_t dim, int32_t region, double Vt, dctx *d,
                       oc_particles *p, int64_t idx, int32_t tauRegionIsValley);
int32_t oci_nvalleys(const oc_model *m);
#endif
