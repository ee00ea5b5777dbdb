// OGPUCheby.cpp -- QDng module libqd-OGPUCheby.so: OCheby's time step on the GB300
// engine (OGPUProp.h).  XML: <propagator name="GPUCheby" ...> with OCheby's
// attributes.
#include "OGPUProp.h"

namespace QDLIB {

class OGPUCheby : public OGPUProp {
 public:
  OGPUCheby() : OGPUProp("OGPUCheby", "Cheby") {}
  virtual Operator *NewInstance() { return new OGPUCheby(); }
};

}  // namespace QDLIB

QDNG_MODULE_OPERATOR_INSTANCE(OGPUCheby)
