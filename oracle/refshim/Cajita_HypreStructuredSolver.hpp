// Part of the Cajita stand-in (oracle reference pin): everything is in Cajita.hpp.
#include <Cajita.hpp>
