/* Header stub used only to compile the reference's CPU sources for the oracle. */
#include "cesa_pcl_compat.h"
