// File formats and program-level entry points of poremaps_gb300: the .inp
// parser, the .raw geometry reader, the field writers, the whole-program run
// and the permeability tensor driver.
#include <fcntl.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "../../include/poremaps.h"
#include "pm_api_internal.h"

using namespace pm;

namespace {

// pwrite the whole buffer at offset 0 without truncating an existing file
// (MPI_File_open with MPI_MODE_RDWR | MPI_MODE_CREATE, output.cc:79).
pm_status write_raw(const std::string& path, const void* data, size_t bytes) {
  int fd = open(path.c_str(), O_RDWR | O_CREAT, 0644);
  if (fd < 0) return set_error(PM_ERR_IO, "cannot open %s for writing", path.c_str());
  const char* p = (const char*)data;
  size_t done = 0;
  while (done < bytes) {
    ssize_t w = pwrite(fd, p + done, bytes - done, (off_t)done);
    if (w <= 0) {
      close(fd);
      return set_error(PM_ERR_IO, "short write to %s", path.c_str());
    }
    done += (size_t)w;
  }
  close(fd);
  return PM_OK;
}

}  // namespace


extern "C" {

// read_problem_params + read_parallel_params (read_problem_params.cc:50-156):
// the 14 keys in fixed order, each pattern read with the same fscanf format.
pm_status pm_read_params(const char* inp_path, pm_params* out) {
  if (!inp_path || !out) return set_error(PM_ERR_INVALID, "bad arguments");
  FILE* f = fopen(inp_path, "r");
  if (!f) return set_error(PM_ERR_IO, "Input file doesnt exist: %s", inp_path);
  pm_params p;
  pm_params_default(&p);
  int n = 0, want = 0;
  want += 3; n += fscanf(f, "dom_decomposition %d %d %d \n", &p.dom_decomposition[0],
                         &p.dom_decomposition[1], &p.dom_decomposition[2]);
  want += 1; n += fscanf(f, "boundary_method %d \n", &p.boundary_method);
  want += 1; n += fscanf(f, "geometry_file_name %399s \n", p.geometry_file_name);
  want += 3; n += fscanf(f, "size_x_y_z %d %d %d \n", &p.size[0], &p.size[1], &p.size[2]);
  want += 1; n += fscanf(f, "voxel_size  %lf \n", &p.voxel_size);
  want += 1; n += fscanf(f, "max_iter %d \n", &p.max_iter);
  want += 1; n += fscanf(f, "it_eval %d \n", &p.it_eval);
  want += 1; n += fscanf(f, "it_write %d \n", &p.it_write);
  want += 1; n += fscanf(f, "log_file_name %399s \n", p.log_file_name);
  want += 1; n += fscanf(f, "solving_algorithm %u \n", &p.solving_algorithm);
  want += 1; n += fscanf(f, "eps %lf \n", &p.eps);
  want += 1; n += fscanf(f, "porosity %lf \n", &p.porosity);
  want += 6; n += fscanf(f, "dom_interest %d %d %d %d %d %d \n", &p.dom_interest[0],
                         &p.dom_interest[1], &p.dom_interest[2], &p.dom_interest[3],
                         &p.dom_interest[4], &p.dom_interest[5]);
  want += 4; n += fscanf(f, "write_output %d %d %d %d \n", &p.write_output[0],
                         &p.write_output[1], &p.write_output[2], &p.write_output[3]);
  fclose(f);
  if (n != want)
    return set_error(PM_ERR_INVALID, "%s: expected %d values in the fixed key order, parsed %d",
                     inp_path, want, n);
  *out = p;
  return PM_OK;
}

// read_geometry (geometry.cc:58-126): headerless uint8, x fastest.
pm_status pm_read_geometry(const char* raw_path, const int size[3], uint8_t* out) {
  if (!raw_path || !size || !out) return set_error(PM_ERR_INVALID, "bad arguments");
  long long n = (long long)size[0] * size[1] * size[2];
  if (n <= 0) return set_error(PM_ERR_INVALID, "bad size");
  FILE* f = fopen(raw_path, "rb");
  if (!f) return set_error(PM_ERR_IO, "cannot open geometry %s", raw_path);
  size_t got = fread(out, 1, (size_t)n, f);
  fclose(f);
  if ((long long)got != n)
    return set_error(PM_ERR_IO, "geometry %s has %zu bytes, expected %lld", raw_path, got, n);
  return PM_OK;
}

// main_stokes_solver.cc:305-411 + write_output_raw / write_domain_decomposition
// (output.cc:53-190): names are prefix + geometry_file_name verbatim.
pm_status pm_write_outputs(pm_problem* pr) {
  if (!pr) return set_error(PM_ERR_INVALID, "bad arguments");
  const pm_params* p = problem_params(pr);
  long long n = problem_nvox(pr);
  std::string g = p->geometry_file_name;
  pm_status s;
  if (p->write_output[2] == 1) {
    std::vector<int32_t> nh((size_t)n);
    if ((s = pm_get_neighborhood(pr, nh.data())) != PM_OK) return s;
    if ((s = write_raw("voxel_neighborhood_" + g, nh.data(), 4 * (size_t)n)) != PM_OK) return s;
  }
  if (p->write_output[1] == 1 || p->write_output[0] == 1) {
    std::vector<double> u, v, w, pp;
    bool vel = p->write_output[0] == 1, prs = p->write_output[1] == 1;
    if (vel) { u.resize(n); v.resize(n); w.resize(n); }
    if (prs) pp.resize(n);
    if ((s = pm_get_fields(pr, vel ? u.data() : nullptr, vel ? v.data() : nullptr,
                           vel ? w.data() : nullptr, prs ? pp.data() : nullptr)) != PM_OK)
      return s;
    if (prs && (s = write_raw("press_" + g, pp.data(), 8 * (size_t)n)) != PM_OK) return s;
    if (vel) {
      double dx = p->voxel_size;
      for (long long i = 0; i < n; ++i) { u[i] *= dx; v[i] *= dx; w[i] *= dx; }
      if ((s = write_raw("velx_" + g, u.data(), 8 * (size_t)n)) != PM_OK) return s;
      if ((s = write_raw("vely_" + g, v.data(), 8 * (size_t)n)) != PM_OK) return s;
      if ((s = write_raw("velz_" + g, w.data(), 8 * (size_t)n)) != PM_OK) return s;
    }
  }
  if (p->write_output[3] == 1) {
    // one device-resident domain: every voxel belongs to rank 0
    std::vector<int32_t> dd((size_t)n, 0);
    if ((s = write_raw("domain_decomp_" + g, dd.data(), 4 * (size_t)n)) != PM_OK) return s;
  }
  return PM_OK;
}

pm_status pm_resume_outputs(pm_problem* pr, int iteration) {
  if (!pr) return set_error(PM_ERR_INVALID, "bad arguments");
  const pm_params* p = problem_params(pr);
  const long long n = problem_nvox(pr);
  const std::string g = p->geometry_file_name;
  const char* pre[4] = {"velx_", "vely_", "velz_", "press_"};
  std::vector<double> f[4];
  for (int k = 0; k < 4; ++k) {
    f[k].resize((size_t)n);
    const std::string name = pre[k] + g;
    FILE* fp = fopen(name.c_str(), "rb");
    if (!fp) return set_error(PM_ERR_IO, "cannot open %s", name.c_str());
    size_t got = fread(f[k].data(), sizeof(double), (size_t)n, fp);
    fclose(fp);
    if (got != (size_t)n) return set_error(PM_ERR_IO, "%s: short file", name.c_str());
  }
  // the writers store velocities times voxel_size
  const double dx = p->voxel_size;
  for (int k = 0; k < 3; ++k)
    for (long long i = 0; i < n; ++i) f[k][i] /= dx;
  return pm_set_fields(pr, f[0].data(), f[1].data(), f[2].data(), f[3].data(), iteration);
}

pm_status pm_run_inp(const char* inp_path, const pm_params* overrides, pm_result* res) {
  pm_params p;
  pm_status s = pm_read_params(inp_path, &p);
  if (s != PM_OK) return s;
  if (overrides) {
    p.order = overrides->order;
    p.precision = overrides->precision;
    p.arith = overrides->arith;
    p.mixed_inner = overrides->mixed_inner;
    p.eps_fixed_point = overrides->eps_fixed_point;
  }
  p.write_log = 1;
  std::vector<uint8_t> geom((size_t)p.size[0] * p.size[1] * p.size[2]);
  if ((s = pm_read_geometry(p.geometry_file_name, p.size, geom.data())) != PM_OK) return s;
  pm_problem* pr = nullptr;
  if ((s = pm_problem_create(&p, geom.data(), &pr)) != PM_OK) return s;
  pm_result r;
  s = pm_solve(pr, &r);
  if (s == PM_OK || s == PM_ERR_NONFINITE) {
    pm_status w = pm_write_outputs(pr);
    if (w != PM_OK) s = w;
  }
  if (res) *res = r;
  pm_problem_destroy(pr);
  return s;
}

// Three axis-rotated solves (README.md:215-227).  Rotation for flow along x:
// new (x', y', z') = old (y, z, x); along y: new (x', y', z') = old (z, x, y).
// Each solve's (wk13, wk23, wk33) is the response along its x', y', z' axes.
pm_status pm_solve_tensor(const pm_params* p, const uint8_t* geom, double K[9],
                          pm_result res3[3]) {
  if (!p || !geom || !K) return set_error(PM_ERR_INVALID, "bad arguments");
  const int nx = p->size[0], ny = p->size[1], nz = p->size[2];
  if (nx < 1 || ny < 1 || nz < 1) return set_error(PM_ERR_INVALID, "bad size");
  pm_params ps[3] = {*p, *p, *p};
  // flow along x: sizes (nx', ny', nz') = (ny, nz, nx); along y: (nz, nx, ny)
  ps[0].size[0] = ny; ps[0].size[1] = nz; ps[0].size[2] = nx;
  ps[1].size[0] = nz; ps[1].size[1] = nx; ps[1].size[2] = ny;
  for (int a = 0; a < 3; ++a) {
    ps[a].write_log = 0;
    memset(ps[a].dom_interest, 0, sizeof(ps[a].dom_interest));
  }
  pm_result r[3];
  pm_status st[3] = {PM_OK, PM_OK, PM_OK};
  std::string err[3];
  // The three solves are independent: each host thread creates its problem
  // (own stream) from the unrotated geometry, which the x and y solves rotate
  // on the device after the upload, and solves it, so the set-up and sweeps
  // of the three axes overlap.
  auto run = [&](int a) {
    pm_problem* pr = nullptr;
    st[a] = problem_create(&ps[a], geom, a < 2 ? a : -1, &pr);
    if (st[a] == PM_OK) st[a] = pm_solve(pr, &r[a]);
    if (st[a] != PM_OK) err[a] = pm_last_error();
    pm_problem_destroy(pr);
  };
  std::vector<std::thread> th;
  for (int a = 0; a < 3; ++a) th.emplace_back(run, a);
  for (auto& t : th) t.join();
  for (int a = 0; a < 3; ++a)
    if (st[a] != PM_OK && st[a] != PM_ERR_NONFINITE) return set_error(st[a], "%s", err[a].c_str());
  // K[3*i + j]: response along axis i to the pressure drop along axis j
  K[3 * 1 + 0] = r[0].wk13; K[3 * 2 + 0] = r[0].wk23; K[3 * 0 + 0] = r[0].wk33;
  K[3 * 2 + 1] = r[1].wk13; K[3 * 0 + 1] = r[1].wk23; K[3 * 1 + 1] = r[1].wk33;
  K[3 * 0 + 2] = r[2].wk13; K[3 * 1 + 2] = r[2].wk23; K[3 * 2 + 2] = r[2].wk33;
  if (res3)
    for (int a = 0; a < 3; ++a) res3[a] = r[a];
  for (int a = 0; a < 3; ++a)
    if (st[a] != PM_OK) return set_error(st[a], "%s", err[a].c_str());
  return PM_OK;
}

}  // extern "C"
