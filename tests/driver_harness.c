/*
 * Test double for the host driver's CPU test: the device entry points the
 * driver calls, backed by the oracle (oracle/nrltb_oracle.c) instead of the
 * GPU, so that nrltb_static's own code -- reading, mode handling, SKENG,
 * SKOUT, QLMT / QAPW and SPNDIR writing -- runs on a machine without a GPU.
 * Test infrastructure only: the product driver links libnrltb_gb300.
 */
#include <stdlib.h>
#include "nrltb.h"

int oracle_bande(const nrltb_structure *st, const nrltb_params *par, const nrltb_kmesh *km,
                 const nrltb_opts *opt, nrltb_result *res, int nthreads);

struct nrltb_ctx { int device; };

int nrltb_ctx_create(nrltb_ctx **out, int device)
{
    *out = (nrltb_ctx *)calloc(1, sizeof **out);
    (*out)->device = device;
    return NRLTB_OK;
}

int nrltb_ctx_destroy(nrltb_ctx *c)
{
    free(c);
    return NRLTB_OK;
}

const char *nrltb_last_error(void) { return "oracle backend"; }

int nrltb_bande(nrltb_ctx *c, const nrltb_structure *st, const nrltb_params *par, const nrltb_kmesh *km,
                const nrltb_opts *opt, nrltb_result *res)
{
    (void)c;
    return oracle_bande(st, par, km, opt, res, 0);
}
