/* The C example of the integration guide (section 2): create a handle for one ddplan row,
 * push one block, count its points.  freqs and block are the caller's. */
#include <stdio.h>
#include "transientx_gb300.h"

int run(const double *freqs, const uint8_t *block)
{
    txg_row row = {0};
    row.td = 1; row.fd = 1; row.bswidth = 0.1f;
    row.nrfi = 2; row.rfi_kind[0] = TXG_RFI_KADANEF; row.rfi_td[0] = 8; row.rfi_fd[0] = 4;
    row.rfi_kind[1] = TXG_RFI_ZDOT;
    row.threKadaneF = 7.f; row.widthlimit = 0.05;
    row.dms = 0; row.ddm = 0.1; row.ndm = 5000; row.minw = 1e-4f; row.maxw = 0.05f;
    row.snrloss = 0.1f; row.thre = 7.f;
    txg_plan plan = {0};
    plan.nchans = 4096; plan.tsamp = 76e-6; plan.frequencies = freqs; plan.ndump = 13156;
    plan.nrows = 1; plan.rows = &row; plan.nbeams = 1; plan.zapthre = 4.f;
    txg_handle *h = NULL;
    int rc = txg_create(&plan, &h);
    if (rc != TXG_OK) {
        fprintf(stderr, "txg_create: %s\n", txg_strerror(rc));
        return rc;
    }
    int64_t n = 0;
    rc = txg_push_block(h, 0, block, 13156);
    if (rc == TXG_OK) rc = txg_sync(h);
    if (rc == TXG_OK) rc = txg_get_candidates(h, 0, 0, NULL, 0, &n);
    txg_destroy(h);
    if (rc != TXG_OK) return rc;
    return (int)n;
}
