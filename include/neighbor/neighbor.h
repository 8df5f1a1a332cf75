// Umbrella header of the neighbor LBVH library for GB300 (sm_103a).
// Same entry point as the reference's include/neighbor/neighbor.h.
#ifndef NEIGHBOR_NEIGHBOR_H_
#define NEIGHBOR_NEIGHBOR_H_

#include "BoundingVolumes.h"
#include "InsertOps.h"
#include "OutputOps.h"
#include "QueryOps.h"
#include "TransformOps.h"
#include "TranslateOps.h"

#include "LBVH.h"
#include "LBVHTraverser.h"
#include "SelfListTuner.h"

#endif // NEIGHBOR_NEIGHBOR_H_
