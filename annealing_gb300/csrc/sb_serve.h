// Continuous-batching request server behind sb_submit / sb_poll / sb_cancel (sb_serve.cpp).
#pragma once
#include <stdint.h>

#include <string>

#include "sb.h"

namespace sbs {
struct Server;
sb_status server_create(Server **out, int device, int64_t hbm_budget, int max_inflight,
                        std::string &err);
void server_destroy(Server *s);
sb_status server_submit(Server *s, const sb_problem *p, const sb_params *prm, uint64_t *ticket);
// err receives the request's error text when it finished with an error
sb_status server_poll(Server *s, uint64_t ticket, sb_result *res, int32_t wait_ms, std::string &err);
sb_status server_cancel(Server *s, uint64_t ticket);
sb_status server_stats(Server *s, sb_serving_stats *out);
}  // namespace sbs
