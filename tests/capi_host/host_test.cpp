// Compiled C++ host of the C ABI: includes include/atm_gb300.h and drives the
// library through the operator wrapper a deal.II maintainer would write (the
// EULEROperator replacement, euler_operator.h:24-211) and the solver calls
// (EulerSolver, Atmospheric_Flow.cc:1100-1257).
//
//   host_test CASE.bin OUT.bin cpu   table checks only; without a device,
//                                    atm_ctx_create must fail with CUDA_ERROR
//   host_test CASE.bin OUT.bin gpu   B p and one IMEX step, results to OUT.bin
//
// CASE.bin (little endian): int32 degree, n_cells, mapping degree, n_inner,
// n_bdry; float64 mapping nodes; int32 inner faces [n_inner][5]; int32
// boundary faces [n_bdry][3]; float64 dt, Ma, Fr, u0; float64 rho, u, p and
// sponge rate per node.  OUT.bin: float64 B p, then rho, u, p after 1 step.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/atm_gb300.h"

namespace {

void check(int rc) {
  if (rc != ATM_OK) throw std::runtime_error(atm_last_error());
}

// device vector with the deal.II Vector accessor the wrapper uses
struct DeviceVec {
  double *ptr = nullptr;
  size_t n = 0;
  explicit DeviceVec(size_t n_) : n(n_) {
    if (cudaMalloc(&ptr, n * sizeof(double)) != cudaSuccess) throw std::runtime_error("cudaMalloc");
  }
  ~DeviceVec() { cudaFree(ptr); }
  DeviceVec(const DeviceVec &) = delete;
  DeviceVec &operator=(const DeviceVec &) = delete;
  double *get_values() const { return ptr; }
  void upload(const double *h) { cudaMemcpy(ptr, h, n * sizeof(double), cudaMemcpyHostToDevice); }
  std::vector<double> download() const {
    std::vector<double> h(n);
    cudaMemcpy(h.data(), ptr, n * sizeof(double), cudaMemcpyDeviceToHost);
    return h;
  }
};

// The operator wrapper of the integration guide, reduced to what is run here.
class GB300EulerOperator {
 public:
  explicit GB300EulerOperator(atm_handle h) : h(h) {}
  void set_dt(double dt) { check(atm_set_dt(h, dt)); }
  void set_Mach(double Ma) { check(atm_set_mach(h, Ma)); }
  void set_Froude(double Fr) { check(atm_set_froude(h, Fr)); }
  void set_HYPERBOLIC_stage(unsigned s) { check(atm_set_hyperbolic_stage(h, (int)s)); }
  void set_NS_stage(unsigned s) { check(atm_set_ns_stage(h, (int)s)); }
  void set_rho_for_fixed(const DeviceVec &v) { check(atm_set_rho_for_fixed(h, v.get_values())); }
  void set_pres_fixed(const DeviceVec &v) { check(atm_set_pres_fixed(h, v.get_values())); }
  void vmult_pressure(DeviceVec &dst, const DeviceVec &src) const {
    check(atm_vmult_pressure(h, dst.get_values(), src.get_values()));
  }

 private:
  atm_handle h;
};

template <typename T>
void read_into(FILE *f, std::vector<T> &v, size_t n) {
  v.resize(n);
  if (n && std::fread(v.data(), sizeof(T), n, f) != n) throw std::runtime_error("short case file");
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: host_test CASE.bin OUT.bin cpu|gpu\n");
    return 2;
  }
  try {
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) throw std::runtime_error("cannot open case file");
    std::vector<int> hdr;
    read_into(f, hdr, 5);
    const int k = hdr[0], nc = hdr[1], m = hdr[2], ni = hdr[3], nb = hdr[4];
    const size_t ns = (size_t)nc * (k + 1) * (k + 1);
    std::vector<double> nodes, par, rho, u, p, alpha;
    std::vector<int> inner, bdry;
    read_into(f, nodes, (size_t)nc * (m + 1) * (m + 1) * 2);
    read_into(f, inner, (size_t)ni * 5);
    read_into(f, bdry, (size_t)nb * 3);
    read_into(f, par, 4);
    read_into(f, rho, ns);
    read_into(f, u, 2 * ns);
    read_into(f, p, ns);
    read_into(f, alpha, ns);
    std::fclose(f);
    const double dt = par[0], Ma = par[1], Fr = par[2], u0 = par[3];

    int n_hanging = -1;
    check(atm_check_mesh(k, nc, m, nodes.data(), ni, inner.data(), nb, bdry.data(), &n_hanging));
    std::printf("mesh ok: %d cells, %d hanging faces\n", nc, n_hanging);

    atm_handle h = nullptr;
    const int rc = atm_ctx_create(2, k, nc, m, nodes.data(), ni, inner.data(), nb, bdry.data(), &h);
    if (std::strcmp(argv[3], "cpu") == 0) {
      int ndev = 0;
      if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        if (rc != ATM_CUDA_ERROR) throw std::runtime_error("context created without a device");
        std::printf("no device: %s\n", atm_last_error());
      } else {
        check(rc);
        check(atm_ctx_destroy(h));
      }
      return 0;
    }
    check(rc);
    std::vector<double> out;
    {
      GB300EulerOperator op(h);
      op.set_dt(dt);
      op.set_Mach(Ma);
      op.set_Froude(Fr);
      op.set_HYPERBOLIC_stage(1);
      op.set_NS_stage(2);
      DeviceVec d_rho(ns), d_p(ns), d_bp(2 * ns);
      d_rho.upload(rho.data());
      d_p.upload(p.data());
      op.set_rho_for_fixed(d_rho);
      op.set_pres_fixed(d_p);
      op.vmult_pressure(d_bp, d_p);
      check(atm_synchronize(h));
      out = d_bp.download();
    }
    check(atm_solver_init(h, dt, Ma, Fr, 1e-10, 30000, 0));
    check(atm_solver_set_state(h, rho.data(), u.data(), p.data()));
    check(atm_solver_set_sponge(h, alpha.data(), u0, 0.0));
    check(atm_solver_run(h, 1));
    check(atm_solver_get_state(h, rho.data(), u.data(), p.data()));
    check(atm_ctx_destroy(h));
    out.insert(out.end(), rho.begin(), rho.end());
    out.insert(out.end(), u.begin(), u.end());
    out.insert(out.end(), p.begin(), p.end());
    FILE *o = std::fopen(argv[2], "wb");
    if (!o || std::fwrite(out.data(), sizeof(double), out.size(), o) != out.size())
      throw std::runtime_error("cannot write output");
    std::fclose(o);
    std::printf("gpu ok\n");
  } catch (const std::exception &e) {
    std::fprintf(stderr, "host_test: %s\n", e.what());
    return 1;
  }
  return 0;
}
