// The reference includes <ATen/ATen.h> beside <torch/extension.h>; nothing
// more is used from it.
#include <torch/extension.h>
