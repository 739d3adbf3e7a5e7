// server.cpp - continuous-batching rollout server (placeholder entry points until the serving
// loop lands; every call reports B2G_E_INVALID_ARG).
#include "../../include/b2g_capi.h"

extern "C" {
B2G_API int b2g_server_create(int, uint64_t, int32_t, float, int32_t, int32_t, b2g_server**) { return B2G_E_INVALID_ARG; }
B2G_API int b2g_server_destroy(b2g_server*) { return B2G_E_INVALID_ARG; }
B2G_API int b2g_server_submit(b2g_server*, uint32_t, int32_t, int32_t, int64_t*) { return B2G_E_INVALID_ARG; }
B2G_API int b2g_server_tick(b2g_server*, int32_t*, double*) { return B2G_E_INVALID_ARG; }
B2G_API int b2g_server_poll(b2g_server*, b2g_request_result*, int32_t, int32_t*) { return B2G_E_INVALID_ARG; }
B2G_API int b2g_server_stats(b2g_server*, int64_t*, int64_t*, int64_t*, int64_t*, int64_t*) { return B2G_E_INVALID_ARG; }
}
