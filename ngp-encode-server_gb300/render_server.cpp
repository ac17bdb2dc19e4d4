// nes_render_server -- runs the GB300 renderer as an instant-ngp-renderer
// endpoint: start it, then start neserver with `--renderer <host>:<port>`
// (src/main.cpp:68-72); neserver's socket_client_thread talks to it unchanged.
//
//   nes_render_server [--port 9000] [--bind 0.0.0.0] [--precision tc|fp32]
//                     [--fov 90] [--seed 0] [--log2-table 19] [--device 0]
#include <csignal>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "nes_gb300.h"

static volatile int g_stop = 0;
static void on_signal(int) { g_stop = 1; }

int main(int argc, char** argv) {
  nes_config cfg;
  nes_config_default(&cfg);
  cfg.precision = NES_PREC_FP16_TC;
  int port = 9000;
  const char* bind_addr = "0.0.0.0";
  for (int i = 1; i + 1 < argc; i += 2) {
    const char* k = argv[i];
    const char* v = argv[i + 1];
    if (!std::strcmp(k, "--port")) port = std::atoi(v);
    else if (!std::strcmp(k, "--bind")) bind_addr = v;
    else if (!std::strcmp(k, "--precision")) cfg.precision = std::strcmp(v, "fp32") ? NES_PREC_FP16_TC : NES_PREC_FP32;
    else if (!std::strcmp(k, "--fov")) cfg.fov_deg = (float)std::atof(v);
    else if (!std::strcmp(k, "--seed")) cfg.seed = std::strtoull(v, nullptr, 10);
    else if (!std::strcmp(k, "--log2-table")) cfg.log2_table_size = (uint32_t)std::atoi(v);
    else if (!std::strcmp(k, "--device")) cfg.device = std::atoi(v);
    else {
      std::fprintf(stderr, "unknown option %s\n", k);
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
  std::fprintf(stderr, "nes_render_server: %llu frames served (%s)\n", (unsigned long long)served,
               rc == NES_OK ? "ok" : nes_strerror(rc));
  nes_destroy(ctx);
  return rc == NES_OK ? 0 : 1;
}
