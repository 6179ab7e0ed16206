/* Drop-in for the reference's holstein/tdvp.h: Holstein::TDVP, State,
 * Operator and parse_stage on libkvgpu (see kv_holstein.h). */
#ifndef KV_HOLSTEIN_TDVP_H
#define KV_HOLSTEIN_TDVP_H
#include "kv_holstein.h"
#endif
