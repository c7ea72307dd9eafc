#include "../ApiSubset.h"
