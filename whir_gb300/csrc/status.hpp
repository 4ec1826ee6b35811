// Status codes shared by the kernels' launch planners and the C ABI: the whir_status enum of the
// public header (WHIR_OK, WHIR_ERR_INVALID, WHIR_ERR_UNSUPPORTED, ...).
#pragma once
#include "../../include/whir_gb300.h"
