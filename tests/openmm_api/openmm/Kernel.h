#include "ApiSubset.h"
