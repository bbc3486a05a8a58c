// Serial Kokkos-subset shim (test infrastructure only).
#include "Kokkos_Core.hpp"
