// sg_internal.h -- shared declarations of the GB300 solve path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/sg_solver.h"

namespace sg {

constexpr int NGLL = 27;    // 3x3x3 GLL points = element nodes
constexpr int NEDOF = 81;   // 3 dofs x 27 nodes
constexpr int NST = 6;      // stress components xx yy zz xy yz zx
constexpr int GEO_STRIDE = 10;  // per GLL point: Jinv (row-major 3x3) + detJ

// Structurally non-zero entries of a 27-node GLL element matrix, upper
// triangle by node blocks: with GLL quadrature at the nodes, nodes that differ
// in all three lattice indices share no quadrature point, so their 3x3 block
// is exactly zero.  The 27 diagonal blocks and the 243 coupled node pairs
// n < m keep their full 3x3 block (row-major, rows of node n): 2430 values
// per element, padded to KS_STRIDE so each element starts on a 64-byte
// boundary in FP32 and FP64.
constexpr int KS_NNZ = 2430;
constexpr int KS_STRIDE = 2432;
constexpr int KS_NBR = 19;  // coupled nodes per node (itself included)

// Fixed reduction geometry (block partials) so that results do not depend on
// the device's SM count or occupancy.
constexpr int NPART = 608;
constexpr int RED_THREADS = 256;

struct Profile {
  bool on = false;
  double ms[8] = {0};
  long long counts[4] = {0};
};

// Deterministic gather of element contributions into global dofs.  Each
// group is one mesh node with at least one free dof: it lists the element
// slots (e*27 + a) that reference the node, in increasing element order (the
// reference's sequential element loop order), and its three dof numbers.
struct GatherTopo {
  int ngroups = 0;
  std::vector<int> ptr, ent, dof;  // host copies
  std::vector<int> pos;            // slot -> position in ent (-1: node with no free dof)
  int *d_ptr = nullptr, *d_ent = nullptr, *d_dof = nullptr, *d_pos = nullptr;
};

// Host-side spectral model (the reference's global arrays).
struct HostMesh {
  int nnode = 0, nelmt = 0, nmatblk = 0, neq = 0;
  std::vector<double> g_coord;   // 3*nnode
  std::vector<int> g_num;        // 27*nelmt (0-based)
  std::vector<int> mat_id;       // nelmt (1-based)
  std::vector<double> gam, ym, nu, phi, coh, psi;
  std::vector<int> gdof;         // 3*nnode
  std::vector<int> gdof_elmt;    // 81*nelmt
  // deck control
  double cg_tol = 1e-12, nl_tol = 1e-12;
  int cg_maxiter = 100, nl_maxiter = 100, phinu = 0, allelastic = 0, nexcav = 0, ninc = 1;
  std::vector<double> srf;
  std::vector<int> excavid, nexcavid;
  int s0_type = -1;
  double z0 = 0, s0 = 0, k0 = 0;
  int iseqload = 0;                       // pseudo-static load (eqload: line)
  double eqkx = 0, eqky = 0, eqkz = 0;
  int iswater = 0;                        // water: line
  std::string wsfile;                     // water-surface file, resolved against the deck's directory
  std::vector<int> water_ids;             // 1-based water material IDs (material list tail)
};

// One record of a water-surface file (src/compute_pressure.f90:61-86): kind 0
// horizontal line, 1 inclined line, 2 meshed faces, the latter listed as
// (0-based element, Exodus face) pairs face[2*(face0+f)], f < nface.
struct WaterSurface {
  int stype, rdir, face0, nface;
  double rx1, rx2, z1, z2;
};
bool read_wsfile(const std::string& path, int nelmt, std::vector<WaterSurface>& surf, std::vector<int>& face,
                 std::string& err);

// host mesh construction (sg_host_mesh.cu)
bool hex2spec(HostMesh& M, int nnode8, const double* x8, const double* y8, const double* z8,
              const int* conn8, std::string& err);
bool apply_bc(HostMesh& M, const int* bc_counts, const int* bc_pairs, std::string& err);
void build_gdof_elmt(HostMesh& M);
bool read_deck(const char* path, HostMesh& M, std::vector<double>& x8, std::vector<double>& y8,
               std::vector<double>& z8, std::vector<int>& conn, std::vector<int>& mid,
               std::vector<double>& props, std::vector<int>& bc_counts, std::vector<int>& bc_pairs,
               std::string& err);
// groups from an element dof map alone (the drop-in has no node ids)
void build_groups_from_gdof(const int* gdof_elmt, int nelmt, int neq, GatherTopo& T);

// sparse symmetric element-matrix layout tables
struct KsTables {
  int nbr[NGLL][KS_NBR];   // lane table: m | kind<<5 | off<<8 ; kind 0 own block, 1 stored (n,m), 2 stored (m,n)
  int entry[KS_NNZ];       // (row, col) of each stored entry: row | col<<8, node(row) <= node(col)
};
const KsTables& ks_tables();

// ---- device tables and setup kernels (sg_kernels.cu) ----
void upload_constants();
void launch_geometry(const double* g_coord, const int* g_num, int nelmt, double* geo, cudaStream_t s);
// K6: element matrices in the sparse symmetric layout; Ydiag receives the
// 81 diagonal entries and Ygrav the gravity load (-detJ*w*gamma on z dofs)
// per element, both gathered later into global vectors.
void launch_stiffness(const double* geo, const int* mat_id, const int* elist, int nel, const double* ym,
                      const double* nu, const double* gam, double* Ks64, float* Ks32, double* Ydiag,
                      double* Ygrav, const int* d_entry, const int* pos, cudaStream_t s,
                      int pseudoeq = 0, double eqkx = 0, double eqky = 0, double eqkz = 0);
void launch_expand_dense(const double* Ks64, int nel, double* dense, const int* d_entry, cudaStream_t s);

}  // namespace sg
