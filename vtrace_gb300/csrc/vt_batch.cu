// vt_batch.cu — batched multi-view rendering (persistent work-stealing kernel, CUDA graph).
#include "vt_api_internal.h"

void vt_batch_release_all() {}
