// Stand-in for src/SiloWriter.hpp (oracle reference pin).  The real writer
// needs the Silo library, which is not available here, and its output is
// not on the per-step path.  This one only remembers the ProblemManager it
// is given (Solver<2> constructs it with its own, src/Solver.hpp:121-122),
// so that the reference driver can read the fields, and counts the writes
// Solver::solve makes.
#ifndef CFREF_SILOWRITER_HPP
#define CFREF_SILOWRITER_HPP

#include <cstdlib>
#include <memory>

namespace CajitaFluids {
namespace refshim {
inline const void*& last_problem_manager() {
    static const void* pm = nullptr;
    return pm;
}
inline int& silo_writes() {
    static int n = 0;
    return n;
}
}  // namespace refshim

template <std::size_t Dims, class ExecutionSpace, class MemorySpace>
class SiloWriter {
  public:
    template <class PM>
    explicit SiloWriter(const std::shared_ptr<PM>& pm) {
        refshim::last_problem_manager() = pm.get();
    }
    void siloWrite(char* name, int, double, double) {
        std::free(name);
        refshim::silo_writes() += 1;
    }
};
}  // namespace CajitaFluids

#endif
