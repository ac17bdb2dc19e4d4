// wire_server.cpp -- a renderer endpoint speaking neserver's renderer
// protocol, so an unmodified neserver can point `--renderer ip:port` at the
// GPU renderer.
//
// Protocol (src/server.cpp:46-60 and 91-112, the client side): each message is
// an 8-byte host-endian size_t length followed by that many bytes; the client
// sends a serialised nesproto::FrameRequest and blocks for a serialised
// nesproto::RenderedFrame (src/server.cpp:161-177).  One request is in flight
// per connection; neserver opens one connection per renderer and reconnects
// every second after a failure (src/server.cpp:216-283).
//
// Each accepted connection gets a thread that loops: read request, render
// through nes_render (the same context serves all connections; calls are
// serialised by the context), write the frame.  A malformed request closes
// the connection, as a failed ParseFromString makes the reference client
// retry (src/server.cpp:174-180); a length above the request limit does too.
#include <arpa/inet.h>
#include <netinet/in.h>
#include <netinet/tcp.h>
#include <poll.h>
#include <sys/socket.h>
#include <unistd.h>

#include <atomic>
#include <cerrno>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "nes_gb300.h"

namespace {

constexpr size_t kMaxRequestBytes = 1 << 20;  // a FrameRequest is ~80 bytes

bool send_all(int fd, const uint8_t* p, size_t n) {
  while (n) {
    const ssize_t r = send(fd, p, n, MSG_NOSIGNAL);
    if (r < 0) {
      if (errno == EINTR || errno == EAGAIN) continue;
      return false;
    }
    p += r;
    n -= (size_t)r;
  }
  return true;
}

// Reads exactly n bytes; false on EOF/error or when *stop becomes nonzero
// while waiting.
bool recv_all(int fd, uint8_t* p, size_t n, const volatile int* stop) {
  while (n) {
    pollfd pf{fd, POLLIN, 0};
    const int pr = poll(&pf, 1, 100);
    if (stop && *stop) return false;
    if (pr == 0) continue;
    if (pr < 0) {
      if (errno == EINTR) continue;
      return false;
    }
    const ssize_t r = recv(fd, p, n, 0);
    if (r == 0) return false;
    if (r < 0) {
      if (errno == EINTR || errno == EAGAIN) continue;
      return false;
    }
    p += r;
    n -= (size_t)r;
  }
  return true;
}

// One connection's thread and the flag it sets when it has ended.
struct Connection {
  std::thread thread;
  std::shared_ptr<std::atomic<bool>> ended;
};

void serve_connection(nes_ctx* ctx, int fd, const volatile int* stop, std::atomic<uint64_t>* served,
                      std::shared_ptr<std::atomic<bool>> ended) {
  int one = 1;
  setsockopt(fd, IPPROTO_TCP, TCP_NODELAY, &one, sizeof(one));
  std::vector<uint8_t> req, frame;
  for (;;) {
    size_t len = 0;  // host-endian size_t, as the reference sends it
    if (!recv_all(fd, reinterpret_cast<uint8_t*>(&len), sizeof(len), stop)) break;
    if (len > kMaxRequestBytes) break;
    req.resize(len);
    if (len && !recv_all(fd, req.data(), len, stop)) break;
    size_t out_len = 0;
    int rc = nes_render(ctx, req.data(), len, nullptr, 0, &out_len);
    if (rc != NES_ENOBUFS) break;  // malformed or unrenderable request
    frame.resize(out_len);
    rc = nes_render(ctx, req.data(), len, frame.data(), frame.size(), &out_len);
    if (rc != NES_OK) break;
    if (!send_all(fd, reinterpret_cast<const uint8_t*>(&out_len), sizeof(out_len)) ||
        !send_all(fd, frame.data(), out_len))
      break;
    served->fetch_add(1);
  }
  close(fd);
  ended->store(true);
}

}  // namespace

extern "C" int nes_tcp_serve(nes_ctx* ctx, const char* bind_addr, uint16_t port, const volatile int* stop,
                             uint16_t* bound_port, uint64_t* frames_served) {
  if (!ctx || !stop) return NES_EINVAL;
  const int lfd = socket(AF_INET, SOCK_STREAM, 0);
  if (lfd < 0) return -errno;
  int one = 1;
  setsockopt(lfd, SOL_SOCKET, SO_REUSEADDR, &one, sizeof(one));
  sockaddr_in addr;
  std::memset(&addr, 0, sizeof(addr));
  addr.sin_family = AF_INET;
  addr.sin_port = htons(port);
  if (inet_pton(AF_INET, bind_addr ? bind_addr : "0.0.0.0", &addr.sin_addr) != 1) {
    close(lfd);
    return NES_EINVAL;
  }
  if (bind(lfd, reinterpret_cast<sockaddr*>(&addr), sizeof(addr)) < 0 || listen(lfd, 16) < 0) {
    const int e = errno;
    close(lfd);
    return -e;
  }
  socklen_t alen = sizeof(addr);
  getsockname(lfd, reinterpret_cast<sockaddr*>(&addr), &alen);
  if (bound_port) *bound_port = ntohs(addr.sin_port);
  std::atomic<uint64_t> served{0};
  std::vector<Connection> conns;
  while (!*stop) {
    // Join the threads of ended connections: clients reconnect after every
    // failure, and an unjoined thread keeps its stack mapped.
    for (size_t i = 0; i < conns.size();) {
      if (conns[i].ended->load()) {
        conns[i].thread.join();
        conns[i] = std::move(conns.back());
        conns.pop_back();
      } else {
        ++i;
      }
    }
    pollfd pf{lfd, POLLIN, 0};
    const int pr = poll(&pf, 1, 100);
    if (pr <= 0) continue;
    const int fd = accept(lfd, nullptr, nullptr);
    if (fd < 0) continue;
    try {
      conns.reserve(conns.size() + 1);  // the push_back below then cannot throw
      auto ended = std::make_shared<std::atomic<bool>>(false);
      std::thread t(serve_connection, ctx, fd, stop, &served, ended);
      conns.push_back(Connection{std::move(t), std::move(ended)});
    } catch (...) {  // no thread (or memory) for this connection: refuse it, keep serving
      close(fd);
    }
  }
  close(lfd);
  for (Connection& c : conns) c.thread.join();
  if (frames_served) *frames_served = served.load();
  return NES_OK;
}
