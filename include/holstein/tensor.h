/* Drop-in for the reference's holstein/tensor.h: Tensor<Rank>, norm, stack,
 * overlap and transpose on libkvgpu (kv_ops.h). */
#ifndef KV_HOLSTEIN_TENSOR_H
#define KV_HOLSTEIN_TENSOR_H
#include "kv_ops.h"
#endif
