// temporary: allocation hooks until the momentum / Poisson modules land
#include "capi_internal.cuh"
namespace ia {
int extra_create(ia_handle*) { return IA_OK; }
void extra_destroy(ia_handle*) {}
}
