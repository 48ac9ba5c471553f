// rt_server.cpp — placeholder (continuous-batching server comes next)
#include "../../include/rt_gb300.h"
extern "C" {
int rt_server_create(rt_ctx *, const rt_server_config *, rt_server **out) { if (out) *out = nullptr; return RT_ERR_INVALID; }
void rt_server_destroy(rt_server *) {}
int rt_server_add_scene(rt_server *, const rt_scene_desc *, int32_t *) { return RT_ERR_INVALID; }
int rt_server_submit(rt_server *, const rt_request *, int64_t *) { return RT_ERR_INVALID; }
int rt_server_step(rt_server *, int32_t *) { return RT_ERR_INVALID; }
int rt_server_drain(rt_server *) { return RT_ERR_INVALID; }
int rt_server_result(rt_server *, int64_t, rt_request_result *, float *) { return RT_ERR_INVALID; }
int rt_server_resident(rt_server *, int32_t, int32_t *) { return RT_ERR_INVALID; }
double rt_server_now(rt_server *) { return 0.0; }
int rt_server_run_poisson(rt_server *, double, double, uint64_t, rt_serve_stats *) { return RT_ERR_INVALID; }
}
