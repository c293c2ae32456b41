// Batched replica boxes (filled in with the persistent replica kernel).
#include "mdg_internal.cuh"
