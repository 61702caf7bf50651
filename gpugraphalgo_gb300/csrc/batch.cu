/*
 * Batched queries (placeholder until the batch engine lands).
 */
#include "ctx.cuh"

struct BatchScratch {};

void ctx_batch_release(gga_ctx *c) { (void)c; }

gga_status gga_msbfs(gga_ctx *, gga_graph *, uint32_t, const uint32_t *, uint32_t *, gga_stats *) {
    return gga_fail(GGA_ERR_UNSUPPORTED, "gga_msbfs not built yet");
}
gga_status gga_sssp_batch(gga_ctx *, gga_graph *, uint32_t, const uint32_t *, uint32_t *, gga_stats *) {
    return gga_fail(GGA_ERR_UNSUPPORTED, "gga_sssp_batch not built yet");
}
gga_status gga_multi_solve(gga_ctx *, uint32_t, const gga_query *, gga_stats *) {
    return gga_fail(GGA_ERR_UNSUPPORTED, "gga_multi_solve not built yet");
}
gga_status gga_server_create(gga_ctx *, uint32_t, gga_graph *const *, uint64_t, uint32_t, gga_server **) {
    return gga_fail(GGA_ERR_UNSUPPORTED, "serving not built yet");
}
gga_status gga_server_submit(gga_server *, uint32_t, gga_algo, uint32_t, uint32_t *, uint64_t *) {
    return gga_fail(GGA_ERR_UNSUPPORTED, "serving not built yet");
}
gga_status gga_server_wait(gga_server *, uint64_t, uint32_t, double *) {
    return gga_fail(GGA_ERR_UNSUPPORTED, "serving not built yet");
}
gga_status gga_server_get_stats(gga_server *, gga_server_stats *) {
    return gga_fail(GGA_ERR_UNSUPPORTED, "serving not built yet");
}
void gga_server_destroy(gga_server *) {}
