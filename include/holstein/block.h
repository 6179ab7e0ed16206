/* Drop-in for the reference's holstein/block.h: Block<Rank> on libkvgpu
 * (kv_ops.h). */
#ifndef KV_HOLSTEIN_BLOCK_H
#define KV_HOLSTEIN_BLOCK_H
#include "kv_ops.h"
#endif
