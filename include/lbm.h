/* lbm.h -- umbrella header, drop-in for lbc include/lbm.h:1-8. */
#ifndef LBM_H
#define LBM_H

#include "lbm_types.h"
#include "lbm_core.h"
#include "lbm_bc.h"
#include "lbm_utils.h"

#endif
