#include "iir_device.cuh"
#include "iir_registry.h"
namespace iirgb {
void register_stcr(std::vector<KernelEntry>&) {}
}
