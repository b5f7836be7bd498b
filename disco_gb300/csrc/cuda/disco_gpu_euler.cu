// Instances of the device path for the Newtonian hydro module (Hydro/euler.c).
#include "instance.cuh"
#include "phys_euler.cuh"

namespace disco_impl {
InstanceBase* make_euler(const disco_host_domain* dom, int precision, int* rc) {
  int nq = dom->num_q;
  if (nq == 5) return precision ? make_instance<Euler<float, 5>, float, 5>(dom, rc)
                                : make_instance<Euler<double, 5>, double, 5>(dom, rc);
  if (nq == 6) return precision ? make_instance<Euler<float, 6>, float, 6>(dom, rc)
                                : make_instance<Euler<double, 6>, double, 6>(dom, rc);
  disco_set_error("euler: NUM_Q must be 5 or 6");
  *rc = DISCO_E_MODULE;
  return nullptr;
}
}  // namespace disco_impl
