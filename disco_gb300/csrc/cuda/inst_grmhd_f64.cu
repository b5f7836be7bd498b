// Instances of the device path for GRMHD (Hydro/grmhd.c on the Schwarzschild
// Kerr-Schild metric, HLL, cell-centred B), plain FP64 (compiled without FMA
// contraction so it rounds like the reference build) arithmetic.
#include "instance.cuh"
#include "phys_grmhd.cuh"

namespace disco_impl {
InstanceBase* make_grmhd_double(const disco_host_domain* dom, int* rc) {
  int nq = dom->num_q;
  if (nq == 8) return make_instance<Grmhd<double, 8>, double, 8>(dom, rc);
  if (nq == 9) return make_instance<Grmhd<double, 9>, double, 9>(dom, rc);
  disco_set_error("grmhd: NUM_Q must be 8 or 9");
  *rc = DISCO_E_MODULE;
  return nullptr;
}
}  // namespace disco_impl
