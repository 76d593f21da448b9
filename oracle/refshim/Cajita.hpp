// Stand-in for the parts of Cajita (Cabana's structured-grid library) that
// cajitafluids' own headers use, so that src/Mesh.hpp, ProblemManager.hpp,
// Interpolation.hpp, TimeIntegrator.hpp, BoundaryConditions.hpp,
// InflowSource.hpp, BodyForce.hpp, VelocityCorrector.hpp and Solver.hpp
// compile unchanged on the host and run one rank of the reference's step.
// TEST INFRASTRUCTURE ONLY (the oracle's reference pin).
//
// Cajita is a third-party dependency (Cabana, version unpinned by the
// reference's spack configs) and is not available here; what this file
// restates is its published semantics on one rank with non-periodic axes
// (the only form src/Mesh.hpp builds, :84-87):
//   - index spaces: ghost depth h; owned cells [h, h+N), owned faces along
//     their normal axis [h, h+N+1); ghosted extents N+2h (+1 along a face's
//     normal axis); local-to-global index = local - h;
//   - the local mesh: entity (i, j) of the ghosted local grid sits at
//     low + (i + o) dx per axis, low = global low corner - h dx, o = 1/2 for
//     a cell axis and 0 along a face's normal axis;
//   - halos: one rank and no periodic axis, so a gather has no neighbour
//     and leaves the ghosts as they are (zero from construction);
//   - B-spline value interpolation of order 1 and 3 (uniform B-splines on
//     the entity's logical coordinate, summed as a tensor product);
//   - ReferenceConjugateGradient: preconditioned CG on the stored 5-point
//     stencil matrix with the stored diagonal preconditioner, x0 = lhs.
// Where Cajita leaves an evaluation order open (the spline sums, the CG dot
// products and updates), this file uses the order the oracle
// (oracle/cf_oracle.c) and the CUDA kernels use, so that all three can be
// compared bit for bit: the spline sum runs along x first with explicit
// fma; dot products are the oracle's blocked canonical order.  HYPRE solvers
// are not available: creating one throws.
#ifndef CFREF_CAJITA_HPP
#define CFREF_CAJITA_HPP

#include <Kokkos_Core.hpp>
#include <mpi.h>

#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace Cajita {

// ---- tags --------------------------------------------------------------
struct Cell {};
struct Node {};
namespace Dim {
enum { I = 0, J = 1, K = 2 };
}
template <int D>
struct Face {};
struct Own {};
struct Ghost {};
struct Local {};
struct Global {};

namespace refshim {
// entity offset along axis d in cell units, and whether the entity has one
// more index than cells along d
template <class E>
struct EntityTraits;
template <>
struct EntityTraits<Cell> {
    static double off(int) { return 0.5; }
    static int extra(int) { return 0; }
};
template <>
struct EntityTraits<Node> {
    static double off(int) { return 0.0; }
    static int extra(int) { return 1; }
};
template <int D>
struct EntityTraits<Face<D>> {
    static double off(int d) { return d == D ? 0.0 : 0.5; }
    static int extra(int d) { return d == D ? 1 : 0; }
};
}  // namespace refshim

// ---- index spaces --------------------------------------------------------
template <std::size_t N>
struct IndexSpace {
    long mn[N], mx[N];
    long min(std::size_t d) const { return mn[d]; }
    long max(std::size_t d) const { return mx[d]; }
    long extent(std::size_t d) const { return mx[d] - mn[d]; }
};

template <class ExecSpace>
Kokkos::MDRangePolicy2 createExecutionPolicy(const IndexSpace<2>& s, const ExecSpace&) {
    Kokkos::MDRangePolicy2 p;
    for (int d = 0; d < 2; ++d) {
        p.lo[d] = s.mn[d];
        p.hi[d] = s.mx[d];
    }
    return p;
}

// ---- meshes and grids ------------------------------------------------------
template <class Scalar, std::size_t NumSpaceDim>
struct UniformMesh {};

template <class MeshType>
class GlobalMesh;

template <class Scalar, std::size_t N>
class GlobalMesh<UniformMesh<Scalar, N>> {
  public:
    GlobalMesh(const std::array<Scalar, N>& low, const std::array<Scalar, N>& high, const std::array<int, N>& num)
        : m_low(low), m_high(high), m_num(num) {
        for (std::size_t d = 0; d < N; ++d) m_cell[d] = (high[d] - low[d]) / num[d];
    }
    Scalar cellSize(std::size_t d) const { return m_cell[d]; }
    Scalar lowCorner(std::size_t d) const { return m_low[d]; }
    Scalar highCorner(std::size_t d) const { return m_high[d]; }
    int globalNumCell(std::size_t d) const { return m_num[d]; }

  private:
    std::array<Scalar, N> m_low, m_high, m_cell;
    std::array<int, N> m_num;
};

template <class Scalar, std::size_t N>
std::shared_ptr<GlobalMesh<UniformMesh<Scalar, N>>> createUniformGlobalMesh(const std::array<Scalar, N>& low,
                                                                            const std::array<Scalar, N>& high,
                                                                            const std::array<int, N>& num) {
    return std::make_shared<GlobalMesh<UniformMesh<Scalar, N>>>(low, high, num);
}

template <std::size_t N>
class BlockPartitioner {
  public:
    virtual ~BlockPartitioner() = default;
};
template <std::size_t N>
class DimBlockPartitioner : public BlockPartitioner<N> {};

template <class MeshType>
class GlobalGrid {
  public:
    GlobalGrid(const std::shared_ptr<GlobalMesh<MeshType>>& mesh) : m_mesh(mesh) {}
    const GlobalMesh<MeshType>& globalMesh() const { return *m_mesh; }
    bool isPeriodic(int) const { return false; }
    int globalOffset(int) const { return 0; }

  private:
    std::shared_ptr<GlobalMesh<MeshType>> m_mesh;
};

template <class MeshType, std::size_t N>
std::shared_ptr<GlobalGrid<MeshType>> createGlobalGrid(MPI_Comm, const std::shared_ptr<GlobalMesh<MeshType>>& mesh,
                                                       const std::array<bool, N>& periodic,
                                                       const BlockPartitioner<N>&) {
    for (std::size_t d = 0; d < N; ++d)
        if (periodic[d]) throw std::runtime_error("Cajita stand-in: periodic axes are not supported");
    return std::make_shared<GlobalGrid<MeshType>>(mesh);
}

template <class MeshType>
class LocalGrid {
  public:
    LocalGrid(const std::shared_ptr<GlobalGrid<MeshType>>& g, int halo) : m_global(g), m_halo(halo) {}
    const GlobalGrid<MeshType>& globalGrid() const { return *m_global; }
    int haloCellWidth() const { return m_halo; }
    template <class E>
    IndexSpace<2> indexSpace(Own, E, Local) const {
        IndexSpace<2> s;
        for (int d = 0; d < 2; ++d) {
            s.mn[d] = m_halo;
            s.mx[d] = m_halo + m_global->globalMesh().globalNumCell(d) + refshim::EntityTraits<E>::extra(d);
        }
        return s;
    }
    template <class E>
    IndexSpace<2> indexSpace(Ghost, E, Local) const {
        IndexSpace<2> s;
        for (int d = 0; d < 2; ++d) {
            s.mn[d] = 0;
            s.mx[d] = 2 * m_halo + m_global->globalMesh().globalNumCell(d) + refshim::EntityTraits<E>::extra(d);
        }
        return s;
    }

  private:
    std::shared_ptr<GlobalGrid<MeshType>> m_global;
    int m_halo;
};

template <class MeshType>
std::shared_ptr<LocalGrid<MeshType>> createLocalGrid(const std::shared_ptr<GlobalGrid<MeshType>>& g, int halo) {
    return std::make_shared<LocalGrid<MeshType>>(g, halo);
}

template <class Device, class MeshType>
class LocalMesh;

template <class Device, class Scalar>
class LocalMesh<Device, UniformMesh<Scalar, 2>> {
  public:
    LocalMesh() = default;
    explicit LocalMesh(const LocalGrid<UniformMesh<Scalar, 2>>& lg) {
        const auto& gm = lg.globalGrid().globalMesh();
        for (int d = 0; d < 2; ++d) {
            m_dx[d] = gm.cellSize(d);
            m_rdx[d] = 1.0 / m_dx[d];
            m_low[d] = gm.lowCorner(d) - (Scalar)lg.haloCellWidth() * m_dx[d];
        }
    }
    template <class E>
    void coordinates(E, const int index[2], Scalar x[2]) const {
        for (int d = 0; d < 2; ++d) {
            Scalar t = (Scalar)index[d] + refshim::EntityTraits<E>::off(d);
            x[d] = m_low[d] + t * m_dx[d];
        }
    }
    Scalar cellSize(int d) const { return m_dx[d]; }
    Scalar rdx(int d) const { return m_rdx[d]; }

  private:
    Scalar m_low[2] = {0, 0}, m_dx[2] = {0, 0}, m_rdx[2] = {0, 0};
};

template <class Device, class MeshType>
LocalMesh<Device, MeshType> createLocalMesh(const LocalGrid<MeshType>& lg) {
    return LocalMesh<Device, MeshType>(lg);
}

// ---- arrays ------------------------------------------------------------------
template <class Entity, class MeshType>
class ArrayLayout {
  public:
    ArrayLayout(const std::shared_ptr<LocalGrid<MeshType>>& lg, int dofs) : m_grid(lg), m_dofs(dofs) {}
    const std::shared_ptr<LocalGrid<MeshType>>& localGrid() const { return m_grid; }
    int dofsPerEntity() const { return m_dofs; }
    IndexSpace<2> indexSpace(Own, Local) const { return m_grid->indexSpace(Own(), Entity(), Local()); }
    IndexSpace<2> indexSpace(Ghost, Local) const { return m_grid->indexSpace(Ghost(), Entity(), Local()); }

  private:
    std::shared_ptr<LocalGrid<MeshType>> m_grid;
    int m_dofs;
};

template <class MeshType, class Entity>
std::shared_ptr<ArrayLayout<Entity, MeshType>> createArrayLayout(const std::shared_ptr<LocalGrid<MeshType>>& lg,
                                                                 int dofs, Entity) {
    return std::make_shared<ArrayLayout<Entity, MeshType>>(lg, dofs);
}

template <class Scalar, class Entity, class MeshType, class MemorySpace>
class Array {
  public:
    using view_type = Kokkos::View<Scalar***, MemorySpace>;
    using layout_type = ArrayLayout<Entity, MeshType>;
    Array(const std::string& label, const std::shared_ptr<layout_type>& layout) : m_layout(layout) {
        IndexSpace<2> g = layout->indexSpace(Ghost(), Local());
        m_view = view_type(label, g.extent(0), g.extent(1), layout->dofsPerEntity());
    }
    view_type view() const { return m_view; }
    const std::shared_ptr<layout_type>& layout() const { return m_layout; }

  private:
    std::shared_ptr<layout_type> m_layout;
    view_type m_view;
};

template <class Scalar, class MemorySpace, class Entity, class MeshType>
std::shared_ptr<Array<Scalar, Entity, MeshType, MemorySpace>> createArray(
    const std::string& label, const std::shared_ptr<ArrayLayout<Entity, MeshType>>& layout) {
    return std::make_shared<Array<Scalar, Entity, MeshType, MemorySpace>>(label, layout);
}

namespace ArrayOp {
template <class A, class Scalar, class Space>
void assign(A& a, const Scalar v, Space) {
    IndexSpace<2> s = a.layout()->indexSpace(Space(), Local());
    auto view = a.view();
    for (std::size_t k = 0; k < view.extent(2); ++k)
        for (long j = s.mn[1]; j < s.mx[1]; ++j)
            for (long i = s.mn[0]; i < s.mx[0]; ++i) view(i, j, k) = v;
}
}  // namespace ArrayOp

namespace IndexConversion {
struct L2G {
    int halo;
    void operator()(const int li, const int lj, int& gi, int& gj) const {
        gi = li - halo;
        gj = lj - halo;
    }
};
template <class MeshType, class Entity>
L2G createL2G(const LocalGrid<MeshType>& lg, Entity) {
    return L2G{lg.haloCellWidth()};
}
}  // namespace IndexConversion

// ---- halos: one rank, no periodic axis -> nothing to exchange -------------------
template <std::size_t N>
struct NodeHaloPattern {};
template <std::size_t N>
struct FaceHaloPattern {};

template <class MemorySpace>
class Halo {
  public:
    template <class ExecSpace, class... Arrays>
    void gather(const ExecSpace&, Arrays&...) const {}
};

template <std::size_t N, class Scalar, class Entity, class MeshType, class MemorySpace, class... Rest>
std::shared_ptr<Halo<MemorySpace>> createHalo(NodeHaloPattern<N>, int,
                                              Array<Scalar, Entity, MeshType, MemorySpace>&, Rest&...) {
    return std::make_shared<Halo<MemorySpace>>();
}

template <class Scalar, class MemorySpace, class Entity, class MeshType, std::size_t N>
std::shared_ptr<Halo<MemorySpace>> createHalo(const ArrayLayout<Entity, MeshType>&, FaceHaloPattern<N>, int) {
    return std::make_shared<Halo<MemorySpace>>();
}

// ---- B-spline interpolation ----------------------------------------------------
// SplineData keeps the point's logical coordinate relative to entity index 0
// of the ghosted local grid; the stencil and weights are formed in
// G2P::value, where the field's extents are known (a trace that leaves the
// ghosted array is clamped to its edge instead of reading past it).
template <class Scalar, std::size_t Order, std::size_t NumSpaceDim, class Entity>
struct SplineData {
    Scalar xi[NumSpaceDim];
};

template <class Device, class Scalar, std::size_t Order, class Entity>
void evaluateSpline(const LocalMesh<Device, UniformMesh<Scalar, 2>>& lm, const Scalar p[2],
                    SplineData<Scalar, Order, 2, Entity>& sd) {
    const int zero[2] = {0, 0};
    Scalar x0[2];
    lm.coordinates(Entity(), zero, x0);
    for (int d = 0; d < 2; ++d) sd.xi[d] = (p[d] - x0[d]) * lm.rdx(d);
}

namespace refshim {
// uniform B-spline weights of order 1 or 3 at logical coordinate xi on an
// axis of ext entities; k0 = first stencil index
template <std::size_t Order>
inline void weights(double xi, long ext, long& k0, double* w) {
    if (Order == 1) {
        xi = std::fmin(std::fmax(xi, 0.0), (double)(ext - 1));
        long k = (long)xi;
        if (k > ext - 2) k = ext - 2;
        double t = xi - (double)k;
        w[0] = 1.0 - t;
        w[1] = t;
        k0 = k;
    } else {
        xi = std::fmin(std::fmax(xi, 1.0), (double)(ext - 2));
        long k = (long)xi;
        if (k > ext - 3) k = ext - 3;
        double t = xi - (double)k;
        double s = 1.0 - t;
        double t2 = t * t;
        double t3 = t2 * t;
        double s3 = (s * s) * s;
        w[0] = s3 * (1.0 / 6.0);
        w[1] = std::fma(0.5, t3, -t2) + (2.0 / 3.0);
        w[2] = std::fma(0.5, (t + t2) - t3, 1.0 / 6.0);
        w[3] = t3 * (1.0 / 6.0);
        k0 = k - 1;
    }
}
}  // namespace refshim

namespace G2P {
template <class View, class Scalar, std::size_t Order, class Entity>
void value(const View& f, const SplineData<Scalar, Order, 2, Entity>& sd, Scalar& out) {
    constexpr int n = Order + 1;
    long kx, ky;
    double wx[4], wy[4];
    refshim::weights<Order>(sd.xi[0], (long)f.extent(0), kx, wx);
    refshim::weights<Order>(sd.xi[1], (long)f.extent(1), ky, wy);
    double val = 0.0;
    for (int b = 0; b < n; ++b) {
        double rs = wx[0] * f(kx, ky + b, 0);
        for (int a = 1; a < n; ++a) rs = std::fma(wx[a], f(kx + a, ky + b, 0), rs);
        val = (b == 0) ? wy[0] * rs : std::fma(wy[b], rs, val);
    }
    out = val;
}
}  // namespace G2P

// ---- the reference conjugate gradient solver --------------------------------------
namespace refshim {
// Canonical dot product over an nx x ny row-major array: units of 64
// columns x 16 rows; lane l of a unit owns columns 2l, 2l+1 and
// accumulates with fma row by row; lanes fold by an xor butterfly
// (16, 8, 4, 2, 1); unit partials go to 256 strided accumulators, folded in
// groups of 32 the same way, the 8 group sums added in order.
inline double fold32(double* s) {
    double tmp[32];
    for (int m = 16; m >= 1; m >>= 1) {
        for (int l = 0; l < 32; ++l) tmp[l] = s[l] + s[l ^ m];
        for (int l = 0; l < 32; ++l) s[l] = tmp[l];
    }
    return s[0];
}

inline double canonical_dot(int nx, int ny, const double* a, const double* b) {
    const int G = (nx + 63) / 64, B = (ny + 15) / 16, U = G * B;
    std::vector<double> partial(U);
    for (int u = 0; u < U; ++u) {
        int g = u % G, band = u / G;
        double lane[32] = {0};
        int j1 = (band + 1) * 16 < ny ? (band + 1) * 16 : ny;
        for (int j = band * 16; j < j1; ++j)
            for (int l = 0; l < 32; ++l) {
                int c = g * 64 + 2 * l;
                if (c < nx) lane[l] = std::fma(a[(std::size_t)j * nx + c], b[(std::size_t)j * nx + c], lane[l]);
                if (c + 1 < nx)
                    lane[l] = std::fma(a[(std::size_t)j * nx + c + 1], b[(std::size_t)j * nx + c + 1], lane[l]);
            }
        partial[u] = fold32(lane);
    }
    double s[256];
    for (int t = 0; t < 256; ++t) {
        s[t] = 0.0;
        for (int u = t; u < U; u += 256) s[t] = s[t] + partial[u];
    }
    double tot = 0.0;
    for (int k = 0; k < 8; ++k) tot = k == 0 ? fold32(s) : tot + fold32(s + 32 * k);
    return tot;
}

// What the last solves did (read by the oracle's reference driver).
struct SolveRecord {
    int iterations;
    int status;  // 0 converged, 1 max_iter, 2 breakdown, 3 NaN
    double bb, rr;
};
inline std::vector<SolveRecord>& solve_log() {
    static std::vector<SolveRecord> log;
    return log;
}
// the owned solution of the last solve, row-major (the pressure, which the
// reference keeps in a private member of its VelocityCorrector)
inline std::vector<double>& last_solution() {
    static std::vector<double> x;
    return x;
}
}  // namespace refshim

template <class Scalar, class Entity, class MeshType, class MemorySpace>
class ReferenceStructuredSolver {
  public:
    using array_type = Array<Scalar, Entity, MeshType, MemorySpace>;
    explicit ReferenceStructuredSolver(const ArrayLayout<Entity, MeshType>& layout)
        : m_layout(std::make_shared<ArrayLayout<Entity, MeshType>>(layout)) {}
    virtual ~ReferenceStructuredSolver() = default;

    void setMatrixStencil(const std::vector<std::array<int, 2>>& stencil, bool) {
        m_stencil = stencil;
        auto lay = std::make_shared<ArrayLayout<Entity, MeshType>>(m_layout->localGrid(), (int)stencil.size());
        m_matrix = std::make_shared<array_type>("matrix", lay);
    }
    const array_type& getMatrixValues() const { return *m_matrix; }
    void setPreconditionerStencil(const std::vector<std::array<int, 2>>& stencil, bool) {
        auto lay = std::make_shared<ArrayLayout<Entity, MeshType>>(m_layout->localGrid(), (int)stencil.size());
        m_precon = std::make_shared<array_type>("preconditioner", lay);
    }
    const array_type& getPreconditionerValues() const { return *m_precon; }
    void setTolerance(double tol) { m_tol = tol; }
    void setMaxIter(int n) { m_maxit = n; }
    void setPrintLevel(int level) { m_print = level; }
    void setup() {}
    int getNumIter() const { return m_iters; }

    // Preconditioned CG from x0 = x on the owned cells, stopping when
    // |r|^2 <= tol^2 |b|^2 (checked before every iteration) or after
    // max_iter iterations.
    virtual void solve(const array_type& b, array_type& x) = 0;

  protected:
    std::shared_ptr<ArrayLayout<Entity, MeshType>> m_layout;
    std::vector<std::array<int, 2>> m_stencil;
    std::shared_ptr<array_type> m_matrix, m_precon;
    double m_tol = 1e-6;
    int m_maxit = 1000, m_print = 0, m_iters = 0;
};

template <class Scalar, class Entity, class MeshType, class MemorySpace>
class ReferenceConjugateGradient : public ReferenceStructuredSolver<Scalar, Entity, MeshType, MemorySpace> {
    using Base = ReferenceStructuredSolver<Scalar, Entity, MeshType, MemorySpace>;

  public:
    using typename Base::array_type;
    using Base::Base;

    void solve(const array_type& b_arr, array_type& x_arr) override {
        IndexSpace<2> own = this->m_layout->indexSpace(Own(), Local());
        const int nx = (int)own.extent(0), ny = (int)own.extent(1);
        const long i0 = own.mn[0], j0 = own.mn[1];
        const std::size_t n = (std::size_t)nx * ny;
        auto A = this->m_matrix->view();
        auto M = this->m_precon->view();
        auto bv = b_arr.view();
        auto xv = x_arr.view();
        std::vector<double> b(n), x(n), r(n), z(n), p(n), q(n);
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                b[(std::size_t)j * nx + i] = bv(i0 + i, j0 + j, 0);
                x[(std::size_t)j * nx + i] = xv(i0 + i, j0 + j, 0);
            }
        // y = A v with the stored stencil entries in stencil order; entries
        // off the owned block read a zero ghost (single rank, no periodic axis)
        auto at = [&](const std::vector<double>& v, int i, int j) {
            if (i < 0 || j < 0 || i >= nx || j >= ny) return 0.0;
            return v[(std::size_t)j * nx + i];
        };
        auto matvec = [&](const std::vector<double>& v, std::vector<double>& y) {
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    double acc = A(i0 + i, j0 + j, 0) * v[(std::size_t)j * nx + i];
                    for (std::size_t e = 1; e < this->m_stencil.size(); ++e)
                        acc = std::fma(A(i0 + i, j0 + j, e),
                                       at(v, i + this->m_stencil[e][0], j + this->m_stencil[e][1]), acc);
                    y[(std::size_t)j * nx + i] = acc;
                }
        };
        matvec(x, q);
        for (std::size_t k = 0; k < n; ++k) r[k] = b[k] - q[k];
        auto minv = [&](std::size_t k) { return M(i0 + (long)(k % nx), j0 + (long)(k / nx), 0); };
        for (std::size_t k = 0; k < n; ++k) z[k] = minv(k) * r[k];
        double rho = refshim::canonical_dot(nx, ny, r.data(), z.data());
        double rr = refshim::canonical_dot(nx, ny, r.data(), r.data());
        double bb = refshim::canonical_dot(nx, ny, b.data(), b.data());
        double beta = 0.0, tol2 = this->m_tol * this->m_tol;
        int it = 0, status = 0;
        if (bb != 0.0) {
            for (;;) {
                if (rr <= tol2 * bb) break;
                if (it >= this->m_maxit) {
                    status = 1;
                    break;
                }
                for (std::size_t c = 0; c < n; ++c) {
                    double zc = minv(c) * r[c];
                    p[c] = it == 0 ? zc : std::fma(beta, p[c], zc);
                }
                matvec(p, q);
                double pq = refshim::canonical_dot(nx, ny, p.data(), q.data());
                if (!(pq > 0.0)) {
                    status = std::isnan(pq) ? 3 : 2;
                    break;
                }
                double alpha = rho / pq, malpha = -alpha;
                for (std::size_t c = 0; c < n; ++c) {
                    x[c] = std::fma(alpha, p[c], x[c]);
                    r[c] = std::fma(malpha, q[c], r[c]);
                    z[c] = minv(c) * r[c];
                }
                double rho_new = refshim::canonical_dot(nx, ny, r.data(), z.data());
                rr = refshim::canonical_dot(nx, ny, r.data(), r.data());
                beta = rho_new / rho;
                rho = rho_new;
                it += 1;
                if (std::isnan(rr)) {
                    status = 3;
                    break;
                }
            }
        }
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) xv(i0 + i, j0 + j, 0) = x[(std::size_t)j * nx + i];
        this->m_iters = it;
        refshim::solve_log().push_back({it, status, bb, rr});
        refshim::last_solution() = x;
    }
};

template <class Scalar, class MemorySpace, class Entity, class MeshType>
std::shared_ptr<ReferenceStructuredSolver<Scalar, Entity, MeshType, MemorySpace>> createReferenceConjugateGradient(
    const ArrayLayout<Entity, MeshType>& layout) {
    return std::make_shared<ReferenceConjugateGradient<Scalar, Entity, MeshType, MemorySpace>>(layout);
}

// HYPRE is not available: the type exists so that the reference's HYPRE
// branch compiles; creating a solver throws.
template <class Scalar, class Entity, class MemorySpace>
class HypreStructuredSolver {
  public:
    template <class... A>
    void setMatrixStencil(const A&...) {}
    template <class A>
    void setMatrixValues(const A&) {}
    void setTolerance(double) {}
    void setMaxIter(int) {}
    void setPrintLevel(int) {}
    void setup() {}
    template <class P>
    void setPreconditioner(const P&) {}
    template <class B, class X>
    void solve(const B&, X&) {
        throw std::runtime_error("HYPRE is not available in the Cajita stand-in");
    }
};

template <class Scalar, class MemorySpace, class Entity, class MeshType>
std::shared_ptr<HypreStructuredSolver<Scalar, Entity, MemorySpace>> createHypreStructuredSolver(
    const std::string& name, const ArrayLayout<Entity, MeshType>&, bool = false) {
    throw std::runtime_error("HYPRE solver '" + name + "' is not available in the Cajita stand-in");
}

}  // namespace Cajita

#endif
