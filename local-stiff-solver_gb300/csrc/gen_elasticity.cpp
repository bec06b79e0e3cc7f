// Synthetic input generator: P1-tetrahedral linear elasticity on a structured
// nx x ny x nz node grid of the unit cube, every hex split into 6 tets along
// its main diagonal (Kuhn / Freudenthal split, conforming across cells).
//
// Host-only helper used to build the benchmark and test matrices (the stiff
// elasticity systems of the workloads); not part of the solve path.
//
// Output: scalar CSR (== CSC, the matrix is symmetric), int32 indices, exact
// zeros pruned.  Dirichlet nodes keep an identity diagonal block so the DOF
// count stays 3 * nx * ny * nz.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

// node linear id offsets of the 15-point stencil, sorted by linear delta
struct Stencil {
    int dx[15], dy[15], dz[15];
};

Stencil make_stencil()
{
    Stencil s;
    int k = 0;
    // neighbours in the Freudenthal triangulation: +/- (sum of a non-empty subset
    // of the unit axes) and the node itself; sort by (dz, dy, dx).
    std::vector<int> off;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                bool pos = dx >= 0 && dy >= 0 && dz >= 0;
                bool neg = dx <= 0 && dy <= 0 && dz <= 0;
                if (!(pos || neg)) continue;
                s.dx[k] = dx; s.dy[k] = dy; s.dz[k] = dz; ++k;
            }
    return s;
}

int slot_of(const Stencil &s, int dx, int dy, int dz)
{
    for (int k = 0; k < 15; ++k)
        if (s.dx[k] == dx && s.dy[k] == dy && s.dz[k] == dz) return k;
    return -1;
}

const int PERM[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};

// local vertex offsets (in cells) of tet p
void tet_vertices(int p, int v[4][3])
{
    v[0][0] = v[0][1] = v[0][2] = 0;
    for (int a = 1; a <= 3; ++a) {
        for (int c = 0; c < 3; ++c) v[a][c] = v[a - 1][c];
        v[a][PERM[p][a - 1]] += 1;
    }
}

// 12x12 stiffness of tet p for E = 1 (row major), spacing h[3], Poisson nu
void tet_stiffness(int p, const double h[3], double nu, double K[144])
{
    int v[4][3];
    tet_vertices(p, v);
    double X[4][3];
    for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 3; ++c) X[a][c] = v[a][c] * h[c];
    double J[3][3];  // columns x_a - x_0
    for (int c = 0; c < 3; ++c)
        for (int a = 0; a < 3; ++a) J[c][a] = X[a + 1][c] - X[0][c];
    double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                 J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                 J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    double inv[3][3];
    inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
    inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
    inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    double g[4][3];  // barycentric gradients: grad(lambda_a) = row a-1 of J^-1
    for (int a = 1; a < 4; ++a)
        for (int c = 0; c < 3; ++c) g[a][c] = inv[a - 1][c];
    for (int c = 0; c < 3; ++c) g[0][c] = -(g[1][c] + g[2][c] + g[3][c]);
    double vol = std::fabs(det) / 6.0;
    double lam = nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    double mu = 1.0 / (2.0 * (1.0 + nu));
    double B[6][12];
    std::memset(B, 0, sizeof(B));
    for (int a = 0; a < 4; ++a) {
        double gx = g[a][0], gy = g[a][1], gz = g[a][2];
        B[0][3 * a + 0] = gx;
        B[1][3 * a + 1] = gy;
        B[2][3 * a + 2] = gz;
        B[3][3 * a + 1] = gz; B[3][3 * a + 2] = gy;
        B[4][3 * a + 0] = gz; B[4][3 * a + 2] = gx;
        B[5][3 * a + 0] = gy; B[5][3 * a + 1] = gx;
    }
    double D[6][6];
    std::memset(D, 0, sizeof(D));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) D[i][j] = lam;
    for (int i = 0; i < 3; ++i) D[i][i] += 2.0 * mu;
    for (int i = 3; i < 6; ++i) D[i][i] = mu;
    for (int r = 0; r < 12; ++r)
        for (int c = 0; c < 12; ++c) {
            double s = 0.0;
            for (int i = 0; i < 6; ++i)
                for (int j = 0; j < 6; ++j) s += B[i][r] * D[i][j] * B[j][c];
            K[r * 12 + c] = vol * s;
        }
}

}  // namespace

extern "C" {

// Assemble.  E_tet[6 * cell + p] is Young's modulus of tet p of cell
// (ci, cj, ck), cell = ci + (nx-1) * (cj + (ny-1) * ck).  Nodes with k == 0 are
// clamped when clamp_z0 != 0.  spring_k is added to the three diagonal entries
// of every node listed in spring_nodes.  The caller provides outer[3N+1] and
// inner/vals of capacity cap (135 * N suffices); the return value is nnz, or -1
// when cap is too small, or -2 on bad arguments.
int64_t lss_gen_elasticity_tet(int32_t nx, int32_t ny, int32_t nz, const double *E_tet, double nu,
                               int32_t clamp_z0, int32_t nspring, const int32_t *spring_nodes,
                               double spring_k, int64_t cap, int32_t *outer, int32_t *inner,
                               double *vals)
{
    if (nx < 2 || ny < 2 || nz < 2) return -2;
    const int64_t N = (int64_t)nx * ny * nz;
    if (3 * N > 0x7fffffffLL) return -2;
    const double h[3] = {1.0 / (nx - 1), 1.0 / (ny - 1), 1.0 / (nz - 1)};
    double Kref[6][144];
    for (int p = 0; p < 6; ++p) tet_stiffness(p, h, nu, Kref[p]);
    const Stencil st = make_stencil();
    // local vertex index of node offset (in cells) inside tet p, -1 if absent
    int vert_of[6][2][2][2];
    for (int p = 0; p < 6; ++p) {
        int v[4][3];
        tet_vertices(p, v);
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int c = 0; c < 2; ++c) vert_of[p][a][b][c] = -1;
        for (int a = 0; a < 4; ++a) vert_of[p][v[a][0]][v[a][1]][v[a][2]] = a;
    }
    std::vector<double> blk((size_t)N * 15 * 9, 0.0);
    std::vector<char> clamped(N, 0);
    if (clamp_z0)
        for (int64_t u = 0; u < (int64_t)nx * ny; ++u) clamped[u] = 1;

#pragma omp parallel for schedule(static)
    for (int64_t u = 0; u < N; ++u) {
        const int i = (int)(u % nx), j = (int)((u / nx) % ny), k = (int)(u / ((int64_t)nx * ny));
        double *B = &blk[(size_t)u * 135];
        for (int ck = k - 1; ck <= k; ++ck)
            for (int cj = j - 1; cj <= j; ++cj)
                for (int ci = i - 1; ci <= i; ++ci) {
                    if (ci < 0 || cj < 0 || ck < 0 || ci >= nx - 1 || cj >= ny - 1 || ck >= nz - 1)
                        continue;
                    const int64_t cell = ci + (int64_t)(nx - 1) * (cj + (int64_t)(ny - 1) * ck);
                    const int lx = i - ci, ly = j - cj, lz = k - ck;
                    for (int p = 0; p < 6; ++p) {
                        const int a = vert_of[p][lx][ly][lz];
                        if (a < 0) continue;
                        const double E = E_tet[6 * cell + p];
                        int v[4][3];
                        tet_vertices(p, v);
                        for (int b = 0; b < 4; ++b) {
                            const int s = slot_of(st, v[b][0] - lx, v[b][1] - ly, v[b][2] - lz);
                            for (int r = 0; r < 3; ++r)
                                for (int c = 0; c < 3; ++c)
                                    B[s * 9 + r * 3 + c] += E * Kref[p][(3 * a + r) * 12 + 3 * b + c];
                        }
                    }
                }
    }
    // Dirichlet: zero rows/cols of clamped nodes, identity diagonal block
#pragma omp parallel for schedule(static)
    for (int64_t u = 0; u < N; ++u) {
        const int i = (int)(u % nx), j = (int)((u / nx) % ny), k = (int)(u / ((int64_t)nx * ny));
        double *B = &blk[(size_t)u * 135];
        for (int s = 0; s < 15; ++s) {
            const int x = i + st.dx[s], y = j + st.dy[s], z = k + st.dz[s];
            if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) continue;
            const int64_t v = x + (int64_t)nx * (y + (int64_t)ny * z);
            if (clamped[u] || clamped[v]) {
                for (int t = 0; t < 9; ++t) B[s * 9 + t] = 0.0;
                if (v == u)
                    for (int t = 0; t < 3; ++t) B[s * 9 + t * 4] = 1.0;
            }
        }
    }
    for (int32_t q = 0; q < nspring; ++q) {
        const int64_t u = spring_nodes[q];
        if (u < 0 || u >= N || clamped[u]) continue;
        const int s0 = slot_of(st, 0, 0, 0);
        for (int t = 0; t < 3; ++t) blk[(size_t)u * 135 + s0 * 9 + t * 4] += spring_k;
    }
    // CSR with pruned exact zeros
    std::vector<int32_t> rowcnt(3 * N + 1, 0);
#pragma omp parallel for schedule(static)
    for (int64_t u = 0; u < N; ++u) {
        const int i = (int)(u % nx), j = (int)((u / nx) % ny), k = (int)(u / ((int64_t)nx * ny));
        const double *B = &blk[(size_t)u * 135];
        for (int r = 0; r < 3; ++r) {
            int32_t c = 0;
            for (int s = 0; s < 15; ++s) {
                const int x = i + st.dx[s], y = j + st.dy[s], z = k + st.dz[s];
                if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) continue;
                for (int cc = 0; cc < 3; ++cc) c += B[s * 9 + r * 3 + cc] != 0.0;
            }
            rowcnt[3 * u + r + 1] = c;
        }
    }
    outer[0] = 0;
    int64_t total = 0;
    for (int64_t q = 0; q < 3 * N; ++q) {
        total += rowcnt[q + 1];
        if (total > 0x7fffffffLL) return -2;
        outer[q + 1] = (int32_t)total;
    }
    if (total > cap) return -1;
#pragma omp parallel for schedule(static)
    for (int64_t u = 0; u < N; ++u) {
        const int i = (int)(u % nx), j = (int)((u / nx) % ny), k = (int)(u / ((int64_t)nx * ny));
        const double *B = &blk[(size_t)u * 135];
        for (int r = 0; r < 3; ++r) {
            int64_t pos = outer[3 * u + r];
            for (int s = 0; s < 15; ++s) {
                const int x = i + st.dx[s], y = j + st.dy[s], z = k + st.dz[s];
                if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) continue;
                const int64_t v = x + (int64_t)nx * (y + (int64_t)ny * z);
                for (int cc = 0; cc < 3; ++cc) {
                    const double a = B[s * 9 + r * 3 + cc];
                    if (a != 0.0) {
                        inner[pos] = (int32_t)(3 * v + cc);
                        vals[pos] = a;
                        ++pos;
                    }
                }
            }
        }
    }
    return total;
}

}  // extern "C"
