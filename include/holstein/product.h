/* Drop-in for the reference's holstein/product.h: product<N1,N2,nc>,
 * apply_zero / apply_single / apply_double and env_sweep on libkvgpu
 * (kv_ops.h). */
#ifndef KV_HOLSTEIN_PRODUCT_H
#define KV_HOLSTEIN_PRODUCT_H
#include "kv_ops.h"
#endif
