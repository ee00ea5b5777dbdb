// OGPUGSPO.cpp -- QDng module libqd-OGPUGSPO.so: OGSPO's time step on the GB300
// engine (OGPUProp.h).  XML: <propagator name="GPUGSPO" ...> with OGSPO's
// attributes.
#include "OGPUProp.h"

namespace QDLIB {

class OGPUGSPO : public OGPUProp {
 public:
  OGPUGSPO() : OGPUProp("OGPUGSPO", "GSPO") {}
  virtual Operator *NewInstance() { return new OGPUGSPO(); }
};

}  // namespace QDLIB

QDNG_MODULE_OPERATOR_INSTANCE(OGPUGSPO)
