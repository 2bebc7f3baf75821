/* openol.h (drop-in) -- umbrella like the reference's include/openol.h:1-22,
 * for the GPU path served by libolgb300.so. */
#ifndef OLGB300_OPENOL_H
#define OLGB300_OPENOL_H
#include "olclass.h"
#include "oldefine.h"
#include "golclass.h"
#include "olprop.h"
#include "olcgh.h"
#include "golprop.h"
#include "golcgh.h"
#include "olobject.h"
#endif
