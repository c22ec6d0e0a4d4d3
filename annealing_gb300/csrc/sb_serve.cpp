// Placeholder until the continuous-batching server lands.
#include "sb_serve.h"
namespace sbs {
struct Server {};
sb_status server_create(Server **, int, int64_t, int, std::string &err) { err = "serving not built"; return SB_ERR_UNSUPPORTED; }
void server_destroy(Server *) {}
sb_status server_submit(Server *, const sb_problem *, const sb_params *, uint64_t *) { return SB_ERR_UNSUPPORTED; }
sb_status server_poll(Server *, uint64_t, sb_result *, int32_t) { return SB_ERR_UNSUPPORTED; }
sb_status server_cancel(Server *, uint64_t) { return SB_ERR_UNSUPPORTED; }
sb_status server_stats(Server *, sb_serving_stats *) { return SB_ERR_UNSUPPORTED; }
}
