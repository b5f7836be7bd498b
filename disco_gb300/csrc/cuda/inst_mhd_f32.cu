// Instances of the device path for Newtonian MHD (Hydro/mhd.c, hlld.c, bfields.c), mixed FP32/FP64 arithmetic.
#include "instance.cuh"
#include "phys_mhd.cuh"

namespace disco_impl {
InstanceBase* make_mhd_float(const disco_host_domain* dom, int* rc) {
  int nq = dom->num_q;
  if (nq == 8) return make_instance<Mhd<float, 8>, float, 8>(dom, rc);
  if (nq == 9) return make_instance<Mhd<float, 9>, float, 9>(dom, rc);
  disco_set_error("mhd: NUM_Q must be 8 or 9");
  *rc = DISCO_E_MODULE;
  return nullptr;
}
}  // namespace disco_impl
