// Instances of the device path for Newtonian hydro (Hydro/euler.c), mixed FP32/FP64 arithmetic.
#include "instance.cuh"
#include "phys_euler.cuh"

namespace disco_impl {
InstanceBase* make_euler_float(const disco_host_domain* dom, int* rc) {
  int nq = dom->num_q;
  if (nq == 5) return make_instance<Euler<float, 5>, float, 5>(dom, rc);
  if (nq == 6) return make_instance<Euler<float, 6>, float, 6>(dom, rc);
  disco_set_error("euler: NUM_Q must be 5 or 6");
  *rc = DISCO_E_MODULE;
  return nullptr;
}
}  // namespace disco_impl
