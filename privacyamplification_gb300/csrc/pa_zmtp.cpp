// pa_zmtp.cpp -- ZMTP 3.0 PUSH/PULL sockets over TCP (the wire the reference's libzmq sockets speak,
// PrivacyAmplification.cu:981-985, 1036-1040, 1147-1153), one peer per socket, NULL security.
//
// Connection: 64-byte greeting (signature FF 00*8 7F, version 3.0, mechanism "NULL", as-server 0,
// filler), then each side sends a READY command carrying its Socket-Type and reads the peer's.  Frames:
// flags (bit 0 MORE, bit 1 LONG size, bit 2 COMMAND), size (1 byte, or 8 bytes big-endian when LONG),
// body.  PING commands (ZMTP 3.1 heartbeats) are answered with PONG; other commands are skipped.
#include "../../include/pa_service.h"

#include <arpa/inet.h>
#include <netdb.h>
#include <netinet/in.h>
#include <netinet/tcp.h>
#include <poll.h>
#include <sys/socket.h>
#include <unistd.h>

#include <atomic>
#include <cerrno>
#include <chrono>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

struct ZSock {
    int type = 0;
    bool bind = false;
    std::string host;
    int port = 0;
    std::atomic<int> lfd{-1};  // listening socket (bind)
    std::atomic<int> fd{-1};   // connected peer
    std::atomic<bool> closed{false};
};

bool parse_endpoint(const char* ep, std::string* host, int* port) {
    std::string s(ep ? ep : "");
    const std::string pre = "tcp://";
    if (s.compare(0, pre.size(), pre) != 0) return false;
    s = s.substr(pre.size());
    size_t c = s.rfind(':');
    if (c == std::string::npos) return false;
    *host = s.substr(0, c);
    *port = std::atoi(s.c_str() + c + 1);
    return *port > 0 && *port < 65536;
}

bool write_all(int fd, const void* p, size_t n) {
    const char* b = static_cast<const char*>(p);
    while (n) {
        ssize_t k = ::send(fd, b, n, MSG_NOSIGNAL);
        if (k < 0 && errno == EINTR) continue;
        if (k <= 0) return false;
        b += k;
        n -= (size_t)k;
    }
    return true;
}

bool read_all(int fd, void* p, size_t n) {
    char* b = static_cast<char*>(p);
    while (n) {
        ssize_t k = ::recv(fd, b, n, 0);
        if (k < 0 && errno == EINTR) continue;
        if (k <= 0) return false;
        b += k;
        n -= (size_t)k;
    }
    return true;
}

bool skip_bytes(int fd, uint64_t n) {
    char tmp[4096];
    while (n) {
        size_t k = n < sizeof(tmp) ? (size_t)n : sizeof(tmp);
        if (!read_all(fd, tmp, k)) return false;
        n -= k;
    }
    return true;
}

bool write_frame(int fd, uint8_t flags, const void* body, uint64_t size) {
    uint8_t hdr[9];
    size_t hl;
    if (size > 255) {
        hdr[0] = flags | 0x02;
        for (int i = 0; i < 8; ++i) hdr[1 + i] = (uint8_t)(size >> (56 - 8 * i));
        hl = 9;
    } else {
        hdr[0] = flags;
        hdr[1] = (uint8_t)size;
        hl = 2;
    }
    return write_all(fd, hdr, hl) && (size == 0 || write_all(fd, body, (size_t)size));
}

bool read_header(int fd, uint8_t* flags, uint64_t* size) {
    if (!read_all(fd, flags, 1)) return false;
    if (*flags & 0x02) {
        uint8_t b[8];
        if (!read_all(fd, b, 8)) return false;
        uint64_t s = 0;
        for (int i = 0; i < 8; ++i) s = (s << 8) | b[i];
        *size = s;
    } else {
        uint8_t b;
        if (!read_all(fd, &b, 1)) return false;
        *size = b;
    }
    return true;
}

const char* type_name(int t) { return t == PA_ZMQ_PUSH ? "PUSH" : "PULL"; }

bool handshake(int fd, int type) {
    uint8_t g[64] = {};
    g[0] = 0xFF;
    g[9] = 0x7F;
    g[10] = 3;  // version 3.0
    g[11] = 0;
    std::memcpy(g + 12, "NULL", 4);
    if (!write_all(fd, g, sizeof(g))) return false;
    uint8_t pg[64];
    if (!read_all(fd, pg, sizeof(pg))) return false;
    if (pg[0] != 0xFF || (pg[9] & 1) == 0 || pg[10] < 3 || std::memcmp(pg + 12, "NULL", 4) != 0) return false;
    // READY with Socket-Type
    const char* tn = type_name(type);
    std::vector<uint8_t> cmd;
    cmd.push_back(5);
    for (const char* c = "READY"; *c; ++c) cmd.push_back((uint8_t)*c);
    const char* pn = "Socket-Type";
    cmd.push_back((uint8_t)std::strlen(pn));
    for (const char* c = pn; *c; ++c) cmd.push_back((uint8_t)*c);
    const uint32_t vl = (uint32_t)std::strlen(tn);
    for (int i = 3; i >= 0; --i) cmd.push_back((uint8_t)(vl >> (8 * i)));
    for (const char* c = tn; *c; ++c) cmd.push_back((uint8_t)*c);
    if (!write_frame(fd, 0x04, cmd.data(), cmd.size())) return false;
    // the peer's READY: check that its socket type pairs with ours
    for (;;) {
        uint8_t fl;
        uint64_t sz;
        if (!read_header(fd, &fl, &sz) || sz > (1u << 20)) return false;
        std::vector<uint8_t> body(sz);
        if (sz && !read_all(fd, body.data(), sz)) return false;
        if (!(fl & 0x04)) return false;  // data before READY
        if (sz < 6 || body[0] != 5 || std::memcmp(body.data() + 1, "READY", 5) != 0) {
            if (sz >= 6 && body[0] == 5 && std::memcmp(body.data() + 1, "ERROR", 5) == 0) return false;
            continue;
        }
        const char* want = type == PA_ZMQ_PUSH ? "PULL" : "PUSH";
        size_t i = 6;
        while (i < sz) {
            size_t nl = body[i++];
            if (i + nl + 4 > sz) return false;
            std::string name(reinterpret_cast<char*>(body.data() + i), nl);
            i += nl;
            uint32_t l = ((uint32_t)body[i] << 24) | ((uint32_t)body[i + 1] << 16) | ((uint32_t)body[i + 2] << 8) | body[i + 3];
            i += 4;
            if (i + l > sz) return false;
            std::string val(reinterpret_cast<char*>(body.data() + i), l);
            i += l;
            if ((name == "Socket-Type" || name == "socket-type") && val != want) return false;
        }
        return true;
    }
}

void drop_peer(ZSock* s) {
    int fd = s->fd.exchange(-1);
    if (fd >= 0) ::close(fd);
}

int resolve(const std::string& host, int port, bool passive, sockaddr_storage* ss, socklen_t* len) {
    addrinfo hints{};
    hints.ai_family = AF_INET;
    hints.ai_socktype = SOCK_STREAM;
    if (passive) hints.ai_flags = AI_PASSIVE;
    addrinfo* res = nullptr;
    const char* h = (host == "*" || host.empty()) ? nullptr : host.c_str();
    std::string ps = std::to_string(port);
    if (getaddrinfo(h, ps.c_str(), &hints, &res) != 0 || !res) return -1;
    std::memcpy(ss, res->ai_addr, res->ai_addrlen);
    *len = res->ai_addrlen;
    freeaddrinfo(res);
    return 0;
}

// Brings up the peer connection (with the handshake); false only once the socket is closed.
bool ensure_peer(ZSock* s) {
    while (s->fd < 0) {
        if (s->closed) return false;
        sockaddr_storage ss;
        socklen_t len = 0;
        if (resolve(s->host, s->port, s->bind, &ss, &len) != 0) {
            std::this_thread::sleep_for(std::chrono::milliseconds(100));
            continue;
        }
        int fd = -1;
        if (s->bind) {
            if (s->lfd < 0) {
                int l = ::socket(AF_INET, SOCK_STREAM, 0);
                int one = 1;
                setsockopt(l, SOL_SOCKET, SO_REUSEADDR, &one, sizeof(one));
                if (l < 0 || ::bind(l, reinterpret_cast<sockaddr*>(&ss), len) != 0 || ::listen(l, 4) != 0) {
                    if (l >= 0) ::close(l);
                    std::this_thread::sleep_for(std::chrono::milliseconds(100));  // the reference retries binds
                    continue;
                }
                s->lfd = l;
            }
            pollfd p{s->lfd, POLLIN, 0};
            int r = ::poll(&p, 1, 100);
            if (r <= 0) continue;
            fd = ::accept(s->lfd, nullptr, nullptr);
            if (fd < 0) continue;
        } else {
            fd = ::socket(AF_INET, SOCK_STREAM, 0);
            if (fd < 0 || ::connect(fd, reinterpret_cast<sockaddr*>(&ss), len) != 0) {
                if (fd >= 0) ::close(fd);
                std::this_thread::sleep_for(std::chrono::milliseconds(100));
                continue;
            }
        }
        int one = 1;
        setsockopt(fd, IPPROTO_TCP, TCP_NODELAY, &one, sizeof(one));
        if (!handshake(fd, s->type)) {
            ::close(fd);
            continue;
        }
        s->fd = fd;
    }
    return true;
}

}  // namespace

// Wakes a thread blocked in send/recv/accept on `sock` (which then returns -1) without freeing it;
// used by the host loop to stop its I/O threads.  Not exported.
void pa_zmtp_interrupt(void* sock) {
    ZSock* s = static_cast<ZSock*>(sock);
    if (!s) return;
    s->closed = true;
    int fd = s->fd.load(), lfd = s->lfd.load();
    if (fd >= 0) ::shutdown(fd, SHUT_RDWR);
    if (lfd >= 0) ::shutdown(lfd, SHUT_RDWR);
}

extern "C" {

int pa_zmq_open(int type, const char* endpoint, int bind, void** sock) {
    if (!sock || (type != PA_ZMQ_PUSH && type != PA_ZMQ_PULL)) return PA_ERR_INVALID_ARG;
    ZSock* s = new ZSock();
    s->type = type;
    s->bind = bind != 0;
    if (!parse_endpoint(endpoint, &s->host, &s->port)) {
        delete s;
        return PA_ERR_INVALID_ARG;
    }
    *sock = s;
    return PA_OK;
}

int64_t pa_zmq_recv(void* sock, void* buf, size_t cap, int* more) {
    ZSock* s = static_cast<ZSock*>(sock);
    if (!s || s->type != PA_ZMQ_PULL) return -1;
    for (;;) {
        if (!ensure_peer(s)) return -1;
        uint8_t fl;
        uint64_t sz;
        if (!read_header(s->fd, &fl, &sz)) {
            drop_peer(s);
            if (s->closed) return -1;
            return -2;  // peer lost: a message in progress is incomplete
        }
        if (fl & 0x04) {  // command
            std::vector<uint8_t> body(sz);
            if (sz > (1u << 20) || (sz && !read_all(s->fd, body.data(), sz))) {
                drop_peer(s);
                return s->closed ? -1 : -2;
            }
            if (sz >= 5 && body[0] == 4 && std::memcmp(body.data() + 1, "PING", 4) == 0) {
                std::vector<uint8_t> pong = {4, 'P', 'O', 'N', 'G'};
                if (sz > 7) pong.insert(pong.end(), body.begin() + 7, body.end());  // echo the context
                write_frame(s->fd, 0x04, pong.data(), pong.size());
            }
            continue;
        }
        const uint64_t take = sz < cap ? sz : cap;
        if ((take && !read_all(s->fd, buf, (size_t)take)) || !skip_bytes(s->fd, sz - take)) {
            drop_peer(s);
            return s->closed ? -1 : -2;
        }
        if (more) *more = (fl & 0x01) ? 1 : 0;
        return (int64_t)sz;
    }
}

int pa_zmq_send(void* sock, const void* buf, size_t len, int more) {
    ZSock* s = static_cast<ZSock*>(sock);
    if (!s || s->type != PA_ZMQ_PUSH) return -1;
    if (!ensure_peer(s)) return -1;
    if (!write_frame(s->fd, more ? 0x01 : 0x00, buf, len)) {
        drop_peer(s);
        return s->closed ? -1 : -2;
    }
    return 0;
}

void pa_zmq_close(void* sock) {
    ZSock* s = static_cast<ZSock*>(sock);
    if (!s) return;
    pa_zmtp_interrupt(s);
    drop_peer(s);
    int lfd = s->lfd.exchange(-1);
    if (lfd >= 0) ::close(lfd);
    delete s;
}

}  // extern "C"
