// OGPUArnoldi.cpp -- QDng module libqd-OGPUArnoldi.so: OArnoldi's time step on the GB300
// engine (OGPUProp.h).  XML: <propagator name="GPUArnoldi" ...> with OArnoldi's
// attributes.
#include "OGPUProp.h"

namespace QDLIB {

class OGPUArnoldi : public OGPUProp {
 public:
  OGPUArnoldi() : OGPUProp("OGPUArnoldi", "Arnoldi") {}
  virtual Operator *NewInstance() { return new OGPUArnoldi(); }
};

}  // namespace QDLIB

QDNG_MODULE_OPERATOR_INSTANCE(OGPUArnoldi)
