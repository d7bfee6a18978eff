// A stand-in for libimmunodbscan_gb300 with the entry points psdbscan calls, so the host's table flow (read, delete empty rows, append results,
// noise removal, write) runs on a machine without a GPU.  Row r gets
// clone_id = r % 3, core = r % 2 and copies = 1 + r % 4 (copies = 7 when the
// parameters ask for the buckets-only candidate path, so the tests can see the
// key arrive); its V call's length is folded into the stats so the tests can
// see the columns arrived.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "immunodbscan_gb300.h"

extern "C" {

idb_status idb_cluster(idb_context *, const idb_input *in, const idb_params *prm, idb_output *out) {
    if (!in || !prm || !out) return IDB_ERR_INVALID_ARG;
    for (uint32_t r = 0; r < in->n_rows; ++r) {
        out->clone_id[r] = r % 3;
        out->core[r] = (int32_t)(r % 2);
        out->copies[r] = prm->candidates == 1 ? 7u : 1 + r % 4;
    }
    if (out->n_uniques) *out->n_uniques = in->n_rows;
    if (out->stats) {
        std::memset(out->stats, 0, sizeof(idb_stats));
        out->stats->n_clusters = in->n_rows ? 2 : 0;
    }
    return IDB_OK;
}

idb_status idb_host_alloc(size_t bytes, void **out) {
    *out = std::malloc(bytes ? bytes : 1);
    return *out ? IDB_OK : IDB_ERR_OUT_OF_MEMORY;
}

idb_status idb_host_free(void *p) {
    std::free(p);
    return IDB_OK;
}

size_t idb_last_error(char *buf, size_t len) {
    if (buf && len) buf[0] = 0;
    return 0;
}

const char *idb_status_string(idb_status s) { return s == IDB_OK ? "ok" : "error"; }

}
