// Pulse critical time step (Domain::getMaximumFrequency, Domain.C:817-945) -- see launch_pulse.
#include "dnl_common.cuh"

namespace dnl {
int launch_pulse(dnl_handle *h, cudaStream_t s)
{
  (void)h;
  (void)s;
  return DNL_ERR_ARG;
}
}  // namespace dnl
