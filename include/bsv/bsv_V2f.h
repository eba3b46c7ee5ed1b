#ifndef BSV_V2F_H
#define BSV_V2F_H
/* Per-type header name used by some bsv callers; everything lives in bsv.h. */
#include "bsv.h"
#endif
