// nes_render_server -- runs the GB300 renderer as an instant-ngp-renderer
// endpoint: start it, then start neserver with `--renderer <host>:<port>`
// (src/main.cpp:68-72); neserver's socket_client_thread talks to it unchanged.
//
//   nes_render_server [--port 9000] [--bind 0.0.0.0] [--precision tc|fp32]
//                     [--fov 90] [--seed 0] [--log2-table 19] [--device 0]
#include <cerrno>
#include <csignal>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "nes_gb300.h"

static volatile int g_stop = 0;
static void on_signal(int) { g_stop = 1; }

// Whole-string integer in [lo, hi].
static bool parse_int(const char* v, long long lo, long long hi, long long* out) {
  char* end = nullptr;
  errno = 0;
  const long long x = std::strtoll(v, &end, 10);
  if (errno || end == v || *end || x < lo || x > hi) return false;
  *out = x;
  return true;
}

int main(int argc, char** argv) {
  nes_config cfg;
  nes_config_default(&cfg);
  cfg.precision = NES_PREC_FP16_TC;
  int port = 9000;
  const char* bind_addr = "0.0.0.0";
  for (int i = 1; i < argc; i += 2) {
    const char* k = argv[i];
    if (i + 1 >= argc) {
      std::fprintf(stderr, "option %s needs a value\n", k);
      return 2;
    }
    const char* v = argv[i + 1];
    long long x = 0;
    bool ok = true;
    if (!std::strcmp(k, "--port")) {
      ok = parse_int(v, 0, 65535, &x);
      port = (int)x;
    } else if (!std::strcmp(k, "--bind")) {
      bind_addr = v;
    } else if (!std::strcmp(k, "--precision")) {
      ok = !std::strcmp(v, "fp32") || !std::strcmp(v, "tc");
      cfg.precision = std::strcmp(v, "fp32") ? NES_PREC_FP16_TC : NES_PREC_FP32;
    } else if (!std::strcmp(k, "--fov")) {
      char* end = nullptr;
      const double f = std::strtod(v, &end);
      ok = end != v && !*end && f > 0.0 && f < 180.0;
      cfg.fov_deg = (float)f;
    } else if (!std::strcmp(k, "--seed")) {
      ok = parse_int(v, 0, 0x7fffffffffffffffll, &x);
      cfg.seed = (uint64_t)x;
    } else if (!std::strcmp(k, "--log2-table")) {
      ok = parse_int(v, 10, 24, &x);
      cfg.log2_table_size = (uint32_t)x;
    } else if (!std::strcmp(k, "--device")) {
      ok = parse_int(v, 0, 1023, &x);
      cfg.device = (int)x;
    } else {
      std::fprintf(stderr, "unknown option %s\n", k);
      return 2;
    }
    if (!ok) {
      std::fprintf(stderr, "bad value for %s: %s\n", k, v);
      return 2;
    }
  }
  nes_ctx* ctx = nullptr;
  int rc = nes_create(&cfg, &ctx);
  if (rc != NES_OK) {
    std::fprintf(stderr, "nes_create: %s\n", nes_strerror(rc));
    return 1;
  }
  std::signal(SIGINT, on_signal);
  std::signal(SIGTERM, on_signal);
  uint16_t bound = 0;
  uint64_t served = 0;
  std::fprintf(stderr, "nes_render_server: listening on %s:%d\n", bind_addr, port);
  rc = nes_tcp_serve(ctx, bind_addr, (uint16_t)port, &g_stop, &bound, &served);
  // Socket failures come back as negative errno values, library errors as NES_E*.
  const char* why = rc == NES_OK ? "ok" : std::strcmp(nes_strerror(rc), "unknown error") ? nes_strerror(rc)
                                                                                        : std::strerror(-rc);
  std::fprintf(stderr, "nes_render_server: %llu frames served (%s)\n", (unsigned long long)served, why);
  nes_destroy(ctx);
  return rc == NES_OK ? 0 : 1;
}
