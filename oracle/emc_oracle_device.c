/* CPU oracle for the ViennaEMC device (2-D) path -- TEST INFRASTRUCTURE ONLY. */
#include "emc_oracle.h"
