#include "CudaSubset.h"
