// OGPUSIL.cpp -- QDng module libqd-OGPUSIL.so: OSIL's time step on the GB300
// engine (OGPUProp.h).  XML: <propagator name="GPUSIL" ...> with OSIL's
// attributes.
#include "OGPUProp.h"

namespace QDLIB {

class OGPUSIL : public OGPUProp {
 public:
  OGPUSIL() : OGPUProp("OGPUSIL", "SIL") {}
  virtual Operator *NewInstance() { return new OGPUSIL(); }
};

}  // namespace QDLIB

QDNG_MODULE_OPERATOR_INSTANCE(OGPUSIL)
