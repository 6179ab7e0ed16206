/* Drop-in for the reference's holstein/svd.h: SVDConfig and
 * svd_impl<R1,R2> on libkvgpu (kv_ops.h). */
#ifndef KV_HOLSTEIN_SVD_H
#define KV_HOLSTEIN_SVD_H
#include "kv_ops.h"
#endif
