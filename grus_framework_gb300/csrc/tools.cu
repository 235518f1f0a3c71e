// tools.cu -- host-side tooling around the traversal core:
//   * grus_convert_edgelist: text edge lists and Matrix Market coordinate
//     files to the Galois v1 .gr layout the loader reads.  The reference's
//     README sends users to Galois' graph-convert for this (README.md:14-27),
//     which is not part of the reference.
//   * grus_save_result: a binary dump of a result array beside the
//     reference's text SaveResults (include/print.cuh:36-45).
//   * grus_telemetry_sample: in-process device telemetry for the server --
//     HBM in use, host-link throughput, clocks, power -- the quantities the
//     reference's tools/pcie.py polls through NVML.  NVML is opened at run
//     time (dlopen), so the library loads on machines without a driver; every
//     query is a read.
#include <dlfcn.h>
#include <nvml.h>

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "grus_internal.cuh"

using namespace grus;

namespace {

struct Edge {
  uint32_t u, v, w;
};

bool blank_or_comment(const char *p) {
  while (*p && std::isspace((unsigned char)*p)) ++p;
  return *p == 0 || *p == '#' || *p == '%';
}

int write_gr(const char *path, uint64_t n, const std::vector<Edge> &e, bool weighted) {
  FILE *f = std::fopen(path, "wb");
  if (!f) {
    set_last_error(std::string("cannot open ") + path + ": " + std::strerror(errno));
    return GRUS_EIO;
  }
  const uint64_t m = e.size();
  const uint64_t h[4] = {1, weighted ? 4ull : 0ull, n, m};
  bool ok = std::fwrite(h, 8, 4, f) == 4;
  std::vector<uint64_t> ends(n, 0);
  for (const Edge &x : e) ++ends[x.u];
  for (uint64_t i = 1; i < n; ++i) ends[i] += ends[i - 1];
  if (ok && n) ok = std::fwrite(ends.data(), 8, n, f) == n;
  std::vector<uint32_t> buf(m);
  for (uint64_t i = 0; i < m; ++i) buf[i] = e[i].v;
  if (ok && m) ok = std::fwrite(buf.data(), 4, m, f) == m;
  if (ok && weighted) {
    if (m % 2) {
      const uint32_t pad = 0;
      ok = std::fwrite(&pad, 4, 1, f) == 1;
    }
    for (uint64_t i = 0; i < m; ++i) buf[i] = e[i].w;
    if (ok && m) ok = std::fwrite(buf.data(), 4, m, f) == m;
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) set_last_error(std::string("write failed: ") + path);
  return ok ? GRUS_OK : GRUS_EIO;
}

// NVML entry points, resolved once.
struct Nvml {
  bool tried = false, ok = false;
  nvmlReturn_t (*init)(void) = nullptr;
  nvmlReturn_t (*by_bus)(const char *, nvmlDevice_t *) = nullptr;
  nvmlReturn_t (*pcie)(nvmlDevice_t, nvmlPcieUtilCounter_t, unsigned int *) = nullptr;
  nvmlReturn_t (*clock)(nvmlDevice_t, nvmlClockType_t, unsigned int *) = nullptr;
  nvmlReturn_t (*power)(nvmlDevice_t, unsigned int *) = nullptr;
  nvmlReturn_t (*temp)(nvmlDevice_t, nvmlTemperatureSensors_t, unsigned int *) = nullptr;
  nvmlReturn_t (*driver)(char *, unsigned int) = nullptr;
};

Nvml &nvml() {
  static Nvml v;
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  if (v.tried) return v;
  v.tried = true;
  void *h = dlopen("libnvidia-ml.so.1", RTLD_NOW | RTLD_LOCAL);
  if (!h) return v;
  v.init = (nvmlReturn_t(*)(void))dlsym(h, "nvmlInit_v2");
  v.by_bus = (nvmlReturn_t(*)(const char *, nvmlDevice_t *))dlsym(h, "nvmlDeviceGetHandleByPciBusId_v2");
  v.pcie = (nvmlReturn_t(*)(nvmlDevice_t, nvmlPcieUtilCounter_t, unsigned int *))dlsym(
      h, "nvmlDeviceGetPcieThroughput");
  v.clock = (nvmlReturn_t(*)(nvmlDevice_t, nvmlClockType_t, unsigned int *))dlsym(
      h, "nvmlDeviceGetClockInfo");
  v.power = (nvmlReturn_t(*)(nvmlDevice_t, unsigned int *))dlsym(h, "nvmlDeviceGetPowerUsage");
  v.temp = (nvmlReturn_t(*)(nvmlDevice_t, nvmlTemperatureSensors_t, unsigned int *))dlsym(
      h, "nvmlDeviceGetTemperature");
  v.driver = (nvmlReturn_t(*)(char *, unsigned int))dlsym(h, "nvmlSystemGetDriverVersion");
  v.ok = v.init && v.by_bus && v.init() == NVML_SUCCESS;
  return v;
}

}  // namespace

extern "C" {

int grus_convert_edgelist(const char *in_path, const char *out_path, uint32_t flags) {
  if (!in_path || !out_path) return GRUS_EINVAL;
  FILE *f = std::fopen(in_path, "r");
  if (!f) {
    set_last_error(std::string("cannot open ") + in_path + ": " + std::strerror(errno));
    return GRUS_ENOENT;
  }
  bool symmetric = flags & GRUS_GEN_SYMMETRIC;
  bool weighted = flags & GRUS_GEN_WEIGHTED;
  bool mm = false, size_line = false;
  uint64_t n = 0;
  std::vector<Edge> e;
  char line[4096];
  uint64_t lineno = 0;
  int rc = GRUS_OK;
  while (std::fgets(line, sizeof(line), f)) {
    ++lineno;
    if (lineno == 1 && std::strncmp(line, "%%MatrixMarket", 14) == 0) {
      std::string hdr(line);
      for (char &c : hdr) c = (char)std::tolower((unsigned char)c);
      if (hdr.find("coordinate") == std::string::npos) {
        set_last_error("Matrix Market: only coordinate format is supported");
        rc = GRUS_EINVAL;
        break;
      }
      mm = true;
      size_line = true;
      if (hdr.find("symmetric") != std::string::npos) symmetric = true;
      if (hdr.find("pattern") != std::string::npos) weighted = false;
      continue;
    }
    if (blank_or_comment(line)) continue;
    if (mm && size_line) {
      unsigned long long r = 0, c = 0, nnz = 0;
      if (std::sscanf(line, "%llu %llu %llu", &r, &c, &nnz) != 3) {
        set_last_error("Matrix Market: bad size line " + std::to_string(lineno));
        rc = GRUS_EINVAL;
        break;
      }
      n = std::max(r, c);
      e.reserve(nnz * (symmetric ? 2 : 1));
      size_line = false;
      continue;
    }
    unsigned long long a = 0, b = 0;
    double wv = 1.0;
    const int got = std::sscanf(line, "%llu %llu %lf", &a, &b, &wv);
    if (got < 2 || (mm && (a == 0 || b == 0))) {
      set_last_error("bad edge at line " + std::to_string(lineno));
      rc = GRUS_EINVAL;
      break;
    }
    if (mm) {
      --a;
      --b;
    }
    if (a >= 0xFFFFFFFEull || b >= 0xFFFFFFFEull || wv < 0 || wv > 4294967295.0) {
      set_last_error("vertex id or weight out of range at line " + std::to_string(lineno));
      rc = GRUS_EOVERFLOW;
      break;
    }
    const uint32_t w = got >= 3 ? (uint32_t)wv : 1u;
    e.push_back({(uint32_t)a, (uint32_t)b, w});
    if (!mm) n = std::max<uint64_t>(n, std::max(a, b) + 1);
  }
  std::fclose(f);
  if (rc) return rc;
  for (const Edge &x : e)
    if (x.u >= n || x.v >= n) {
      set_last_error("edge endpoint beyond the declared matrix size");
      return GRUS_EINVAL;
    }
  if (symmetric) {
    const size_t m0 = e.size();
    for (size_t i = 0; i < m0; ++i)
      if (e[i].u != e[i].v) e.push_back({e[i].v, e[i].u, e[i].w});
  }
  std::sort(e.begin(), e.end(), [](const Edge &x, const Edge &y) {
    return std::tie(x.u, x.v, x.w) < std::tie(y.u, y.v, y.w);
  });
  if (symmetric) {
    // both directions may have been listed: keep one (u, v), the lightest
    e.erase(std::unique(e.begin(), e.end(),
                        [](const Edge &x, const Edge &y) { return x.u == y.u && x.v == y.v; }),
            e.end());
  }
  return write_gr(out_path, n, e, weighted);
}

int grus_save_result(const char *path, const void *values, uint64_t n, uint32_t type) {
  if (!path || (!values && n) || type > GRUS_RESULT_F32) return GRUS_EINVAL;
  std::vector<uint32_t> host;
  const void *src = values;
  if (n && is_device_pointer(values)) {
    host.resize(n);
    GRUS_CUDA_TRY(cudaMemcpy(host.data(), values, n * 4, cudaMemcpyDeviceToHost));
    src = host.data();
  }
  FILE *f = std::fopen(path, "wb");
  if (!f) {
    set_last_error(std::string("cannot open ") + path + ": " + std::strerror(errno));
    return GRUS_EIO;
  }
  const char magic[8] = {'G', 'R', 'U', 'S', 'R', 'E', 'S', '1'};
  const uint32_t t[2] = {type, 4u};
  bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(t, 4, 2, f) == 2 &&
            std::fwrite(&n, 8, 1, f) == 1;
  if (ok && n) ok = std::fwrite(src, 4, n, f) == n;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GRUS_OK : GRUS_EIO;
}

int grus_telemetry_sample(grus_telemetry *out) {
  if (!out) return GRUS_EINVAL;
  std::memset(out, 0, sizeof(*out));
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
    out->hbm_free_bytes = free_b;
    out->hbm_total_bytes = total_b;
    out->valid |= GRUS_TEL_HBM;
  } else {
    cudaGetLastError();
    set_last_error("no CUDA device visible");
    return GRUS_ENODEV;
  }
  Nvml &v = nvml();
  if (!v.ok) return GRUS_OK;  // device memory only
  int dev = 0;
  char bus[32] = {0};
  nvmlDevice_t h;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetPCIBusId(bus, sizeof(bus), dev) != cudaSuccess ||
      v.by_bus(bus, &h) != NVML_SUCCESS) {
    cudaGetLastError();
    return GRUS_OK;
  }
  unsigned int a = 0, b = 0;
  if (v.pcie && v.pcie(h, NVML_PCIE_UTIL_TX_BYTES, &a) == NVML_SUCCESS &&
      v.pcie(h, NVML_PCIE_UTIL_RX_BYTES, &b) == NVML_SUCCESS) {
    out->link_tx_kbps = a;
    out->link_rx_kbps = b;
    out->valid |= GRUS_TEL_LINK;
  }
  if (v.clock && v.clock(h, NVML_CLOCK_SM, &a) == NVML_SUCCESS &&
      v.clock(h, NVML_CLOCK_MEM, &b) == NVML_SUCCESS) {
    out->sm_clock_mhz = a;
    out->mem_clock_mhz = b;
    out->valid |= GRUS_TEL_CLOCKS;
  }
  if (v.power && v.power(h, &a) == NVML_SUCCESS) {
    out->power_mw = a;
    out->valid |= GRUS_TEL_POWER;
  }
  if (v.temp && v.temp(h, NVML_TEMPERATURE_GPU, &a) == NVML_SUCCESS) {
    out->temperature_c = a;
    out->valid |= GRUS_TEL_TEMP;
  }
  if (v.driver && v.driver(out->driver_version, sizeof(out->driver_version)) == NVML_SUCCESS)
    out->valid |= GRUS_TEL_DRIVER;
  return GRUS_OK;
}

}  // extern "C"
