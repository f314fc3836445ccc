/*
 * KDTree.h -- lets unmodified NBodylib sources that `#include <KDTree.h>` (for example
 * src/Analysis/Density.cxx, DensitySmooth) build against the GPU drop-in: put this
 * directory ahead of NBodylib's src/KDTree on the include path.
 */
#pragma once
#include "../nbkdt/KDTree.h"
