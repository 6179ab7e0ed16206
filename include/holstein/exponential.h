/* Drop-in for the reference's holstein/exponential.h: KrylovConfig,
 * KrylovExit and local_krylov<Rank> on libkvgpu (kv_ops.h). */
#ifndef KV_HOLSTEIN_EXPONENTIAL_H
#define KV_HOLSTEIN_EXPONENTIAL_H
#include "kv_ops.h"
#endif
