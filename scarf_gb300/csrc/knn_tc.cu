// a6/a7, precision form: BF16 distance tiles on the tcgen05 tensor cores.
#include "common.cuh"
