// Stand-in for Cabana's umbrella header (oracle reference pin; the
// cajitafluids headers include it but use only Cajita).
#ifndef CFREF_CABANA_CORE_HPP
#define CFREF_CABANA_CORE_HPP
#include <Kokkos_Core.hpp>
#endif
