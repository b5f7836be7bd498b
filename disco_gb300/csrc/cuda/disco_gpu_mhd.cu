// Instances of the device path for the Newtonian MHD module (Hydro/mhd.c,
// hlld.c, bfields.c constrained transport).
#include "instance.cuh"
#include "phys_mhd.cuh"

namespace disco_impl {
InstanceBase* make_mhd(const disco_host_domain* dom, int precision, int* rc) {
  int nq = dom->num_q;
  if (nq == 8) return precision ? make_instance<Mhd<float, 8>, float, 8>(dom, rc)
                                : make_instance<Mhd<double, 8>, double, 8>(dom, rc);
  if (nq == 9) return precision ? make_instance<Mhd<float, 9>, float, 9>(dom, rc)
                                : make_instance<Mhd<double, 9>, double, 9>(dom, rc);
  disco_set_error("mhd: NUM_Q must be 8 or 9");
  *rc = DISCO_E_MODULE;
  return nullptr;
}
}  // namespace disco_impl
