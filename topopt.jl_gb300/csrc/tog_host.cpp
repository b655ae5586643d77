// Host-side set-up of libtopopt_gb300: grid numbering, element stiffness,
// modal operator and filter stencil.  Pure C++ (no CUDA calls), so these
// functions are usable and testable without a GPU.
#include "tog_host.h"

#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace tog {

static const int kHexCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                     {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
static const int kQuadCorner[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};

void grid_counts(int dim, const int32_t* nel, long long* nnodes, long long* ncells) {
    long long nn = 1, nc = 1;
    for (int d = 0; d < dim; ++d) {
        nn *= (long long)nel[d] + 1;
        nc *= nel[d];
    }
    *nnodes = nn;
    *ncells = nc;
}

// Ferrite DofHandler numbering for one Lagrange^dim field on a structured grid
// (TopOpt.jl src/TopOptProblems/metadata.jl:116-145 reads it back): cells are
// visited in order (x fastest), their vertices in Ferrite's local order, and
// every node seen for the first time receives `dim` consecutive dofs.
// node_dofs[n*dim + c] is the 0-based dof of component c of lexicographic node n.
void node_dofs_first_touch(int dim, const int32_t* nel, int32_t* node_dofs) {
    long long nnodes, ncells;
    grid_counts(dim, nel, &nnodes, &ncells);
    const long long nnx = nel[0] + 1, nny = nel[1] + 1;
    for (long long i = 0; i < nnodes * dim; ++i) node_dofs[i] = -1;
    int32_t next = 0;
    const int nv = dim == 2 ? 4 : 8;
    const int nez = dim == 3 ? nel[2] : 1;
    for (int k = 0; k < nez; ++k)
        for (int j = 0; j < nel[1]; ++j)
            for (int i = 0; i < nel[0]; ++i)
                for (int a = 0; a < nv; ++a) {
                    long long n;
                    if (dim == 2)
                        n = (i + kQuadCorner[a][0]) + nnx * (j + kQuadCorner[a][1]);
                    else
                        n = (i + kHexCorner[a][0]) + nnx * ((j + kHexCorner[a][1]) + nny * (k + kHexCorner[a][2]));
                    if (node_dofs[n * dim] < 0) {
                        for (int c = 0; c < dim; ++c) node_dofs[n * dim + c] = next + c;
                        next += dim;
                    }
                }
}

// cell_dofs[e*ndpc + dim*a + c] (metadata.jl:40-50): dof of component c of
// Ferrite-local vertex a of cell e.
void cell_dofs_from_node_dofs(int dim, const int32_t* nel, const int32_t* node_dofs, int32_t* cell_dofs) {
    const long long nnx = nel[0] + 1, nny = nel[1] + 1;
    const int nv = dim == 2 ? 4 : 8;
    const int ndpc = nv * dim;
    const int nez = dim == 3 ? nel[2] : 1;
    long long e = 0;
    for (int k = 0; k < nez; ++k)
        for (int j = 0; j < nel[1]; ++j)
            for (int i = 0; i < nel[0]; ++i, ++e)
                for (int a = 0; a < nv; ++a) {
                    long long n;
                    if (dim == 2)
                        n = (i + kQuadCorner[a][0]) + nnx * (j + kQuadCorner[a][1]);
                    else
                        n = (i + kHexCorner[a][0]) + nnx * ((j + kHexCorner[a][1]) + nny * (k + kHexCorner[a][2]));
                    for (int c = 0; c < dim; ++c) cell_dofs[e * ndpc + dim * a + c] = node_dofs[n * dim + c];
                }
}

// Ke_ab = sum_q dotdot(grad phi_a, C, grad phi_b) dOmega, Gauss-Legendre with 4
// points per direction (TopOpt.jl matrices_and_vectors.jl:68-177,
// solvers_api.jl:432-444), Lame constants of matrices_and_vectors.jl:83-84
// (plane strain in 2D; plane_stress = 1 selects lambda* = 2 lambda mu/(lambda+2mu)).
// Output in Ferrite dof order dim*a + c, row-major (the matrix is symmetric).
void element_stiffness(int dim, const double* size, double E, double nu, int plane_stress, double* Ke) {
    double lam = E * nu / ((1 + nu) * (1 - 2 * nu));
    const double mu = E / (2 * (1 + nu));
    if (plane_stress) lam = 2 * lam * mu / (lam + 2 * mu);
    // 4-point Gauss-Legendre nodes / weights
    const double gp[4] = {-0.8611363115940526, -0.3399810435848563, 0.3399810435848563, 0.8611363115940526};
    const double gw[4] = {0.3478548451374538, 0.6521451548625461, 0.6521451548625461, 0.3478548451374538};
    const int nv = dim == 2 ? 4 : 8;
    const int nd = nv * dim;
    for (int i = 0; i < nd * nd; ++i) Ke[i] = 0.0;
    double detJ = 1.0;
    for (int d = 0; d < dim; ++d) detJ *= size[d] / 2.0;
    const int nq = dim == 2 ? 16 : 64;
    for (int q = 0; q < nq; ++q) {
        int qi[3] = {q % 4, (q / 4) % 4, q / 16};
        double xi[3], w = 1.0;
        for (int d = 0; d < dim; ++d) {
            xi[d] = gp[qi[d]];
            w *= gw[qi[d]];
        }
        double g[8][3];
        for (int a = 0; a < nv; ++a) {
            double ref[3];
            for (int d = 0; d < dim; ++d) ref[d] = 2.0 * (dim == 2 ? kQuadCorner[a][d] : kHexCorner[a][d]) - 1.0;
            for (int d = 0; d < dim; ++d) {
                double v = ref[d] / 2.0;
                for (int e = 0; e < dim; ++e)
                    if (e != d) v *= (1.0 + ref[e] * xi[e]) / 2.0;
                g[a][d] = v * 2.0 / size[d];
            }
        }
        const double dO = detJ * w;
        for (int a = 0; a < nv; ++a)
            for (int b = 0; b < nv; ++b) {
                double dot = 0.0;
                for (int d = 0; d < dim; ++d) dot += g[a][d] * g[b][d];
                for (int i = 0; i < dim; ++i)
                    for (int j = 0; j < dim; ++j) {
                        const double v = lam * g[a][i] * g[b][j] + mu * ((i == j ? dot : 0.0) + g[a][j] * g[b][i]);
                        Ke[(dim * a + i) * nd + (dim * b + j)] += v * dO;
                    }
            }
    }
}

// Modal operator: M = T Ke T' / 4^dim with T the Hadamard transform of the
// corner values (corner n = bx + 2 by + 4 bz).  Throws if Ke has entries
// outside the block structure (never for a rectangular isotropic element).
template <int DIM>
static void modal_from_ke(const double* KeF, ModalD<DIM>& M, double* kd) {
    constexpr int NC = 1 << DIM;
    constexpr int ND = NC * DIM;
    // Ke in corner order
    double K[ND][ND];
    const int* f2c = kFerriteToCorner;
    for (int a = 0; a < NC; ++a)
        for (int b = 0; b < NC; ++b)
            for (int i = 0; i < DIM; ++i)
                for (int j = 0; j < DIM; ++j)
                    K[f2c[a] * DIM + i][f2c[b] * DIM + j] = KeF[(DIM * a + i) * ND + (DIM * b + j)];
    double T[NC][NC];
    for (int m = 0; m < NC; ++m)
        for (int n = 0; n < NC; ++n) {
            double v = 1.0;
            for (int d = 0; d < DIM; ++d)
                if ((m >> d) & 1) v *= ((n >> d) & 1) ? 1.0 : -1.0;
            T[m][n] = v;
        }
    // Mm[(m,c),(n,d)] = sum_{a,b} T[m][a] K[(a,c),(b,d)] T[n][b] / NC^2
    static thread_local double Mm[ND][ND];
    double mx = 0.0;
    for (int m = 0; m < NC; ++m)
        for (int c = 0; c < DIM; ++c)
            for (int n = 0; n < NC; ++n)
                for (int d = 0; d < DIM; ++d) {
                    double s = 0.0;
                    for (int a = 0; a < NC; ++a)
                        for (int b = 0; b < NC; ++b) s += T[m][a] * K[a * DIM + c][b * DIM + d] * T[n][b];
                    s /= (double)(NC * NC);
                    Mm[m * DIM + c][n * DIM + d] = s;
                    mx = std::fmax(mx, std::fabs(s));
                }
    std::memset(&M, 0, sizeof(M));
    for (int m = 0; m < NC; ++m)
        for (int c = 0; c < DIM; ++c)
            for (int n = 0; n < NC; ++n)
                for (int d = 0; d < DIM; ++d) {
                    const double v = Mm[m * DIM + c][n * DIM + d];
                    bool structural = false;
                    if (m != 0 && n == m && d == c) {
                        M.D[m][c] = v;
                        structural = true;
                    } else if (m != 0 && d != c && (((m >> c) & 1) != ((m >> d) & 1)) && n == (m ^ (1 << c) ^ (1 << d))) {
                        M.O[m][c][d] = v;
                        structural = true;
                    }
                    if (!structural && std::fabs(v) > 1e-12 * mx)
                        throw std::runtime_error("element stiffness is not block-structured in the modal basis");
                }
    for (int c = 0; c < DIM; ++c) {
        kd[c] = K[c][c];
        for (int a = 1; a < NC; ++a)
            if (std::fabs(K[a * DIM + c][a * DIM + c] - kd[c]) > 1e-12 * std::fabs(kd[c]))
                throw std::runtime_error("element stiffness diagonal differs between corners");
    }
}

void modal_operator(int dim, const double* KeF, double* D_out, double* O_out, double* kd) {
    if (dim == 3) {
        ModalD<3> M;
        modal_from_ke<3>(KeF, M, kd);
        std::memcpy(D_out, M.D, sizeof(M.D));
        std::memcpy(O_out, M.O, sizeof(M.O));
    } else {
        ModalD<2> M;
        modal_from_ke<2>(KeF, M, kd);
        std::memcpy(D_out, M.D, sizeof(M.D));
        std::memcpy(O_out, M.O, sizeof(M.O));
    }
}

// Filter stencil of the node-based filter (TopOpt.jl CheqFilters.jl:66-118):
// every node at distance d < rmin from the cell centre (mean of the corner
// coordinates) carries the weight rmin - d.  The reference pushes such a node
// once per cell that holds it, which the kernels apply as a valence factor.
// Offsets are relative to the cell's lower corner node.
int filter_stencil(int dim, const double* size, double rmin, std::vector<int>& off, std::vector<double>& w) {
    off.clear();
    w.clear();
    int R[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) R[d] = (int)std::ceil(rmin / size[d]) + 1;
    const int zlo = dim == 3 ? -R[2] : 0, zhi = dim == 3 ? R[2] + 1 : 0;
    for (int dz = zlo; dz <= zhi; ++dz)
        for (int dy = -R[1]; dy <= R[1] + 1; ++dy)
            for (int dx = -R[0]; dx <= R[0] + 1; ++dx) {
                const int o[3] = {dx, dy, dz};
                double s2 = 0.0;
                for (int d = 0; d < dim; ++d) {
                    // node coordinate minus centre, both in the coordinates of a cell at the origin
                    const double node = o[d] * size[d];
                    const double centre = (0.0 + size[d]) / 2.0;
                    s2 += (node - centre) * (node - centre);
                }
                const double dist = std::sqrt(s2);
                if (dist < rmin) {
                    off.push_back(dx);
                    off.push_back(dy);
                    off.push_back(dz);
                    w.push_back(std::fmax(rmin - dist, 0.0));
                }
            }
    return (int)w.size();
}

}  // namespace tog
