// Stand-in declaration for compiling flecsolve's finite-volume physics
// operators (flecsolve/physics/) without FleCSI.  See interface.hh.
#pragma once
#include "flecsi/topo/narray/interface.hh"
