// pa_service.cpp -- the host loop: seeds and keys in, privacy-amplified blocks out.
//
// Mirrors the reference's main() + mainloop() + I/O threads (PrivacyAmplification.cu:1394-1680,
// 1686-2118, 969-1225) around the GB300 engine:
//   seed thread   PULL address_seed_in: message {int32 reuse_seed_amount, n/8 seed bytes} (:999-1000),
//                 or toeplitz_seed_path read once (:895-925, exit 103/104);
//   key thread    PULL address_key_in: message {bool do_xor_key_rest, bool do_compress, uint32
//                 vertical_block, data} with data = recv_key (n/32+1 words, split by key2StartRest)
//                 when do_xor, else key_start (h/32+1 words) (:1055-1077); or keyfile_path (:928-966,
//                 exit 105/106);
//   main thread   per block: a new seed when the previous one is used up (reuse_seed_amount rule,
//                 :1769-1797, 2099-2101), then pa_process;
//   sender        verify SHA3-256 of the v/8 result bytes (exit 101, :1130-1140), store the first
//                 results in a file (:1162-1178), PUSH to address_amp_out (:1180-1190).
// Queues between the threads hold input_blocks_to_cache / output_blocks_to_cache entries, the
// reference's ring-buffer depths.
#include "../../include/pa_service.h"

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

void pa_zmtp_interrupt(void* sock);  // pa_zmtp.cpp

namespace {

template <class T>
class BoundedQueue {
public:
    explicit BoundedQueue(size_t cap) : cap_(cap ? cap : 1) {}
    bool push(T v) {
        std::unique_lock<std::mutex> l(m_);
        cv_.wait(l, [&] { return closed_ || q_.size() < cap_; });
        if (closed_) return false;
        q_.push_back(std::move(v));
        cv_.notify_all();
        return true;
    }
    bool pop(T* v) {
        std::unique_lock<std::mutex> l(m_);
        cv_.wait(l, [&] { return closed_ || !q_.empty(); });
        if (q_.empty()) return false;
        *v = std::move(q_.front());
        q_.pop_front();
        cv_.notify_all();
        return true;
    }
    void close() {
        std::lock_guard<std::mutex> l(m_);
        closed_ = true;
        cv_.notify_all();
    }

private:
    size_t cap_;
    bool closed_ = false;
    std::deque<T> q_;
    std::mutex m_;
    std::condition_variable cv_;
};

struct SeedMsg {
    int32_t reuse = 0;
    std::vector<uint32_t> words;
};

struct KeyMsg {
    uint32_t v = 0, flags = 0;
    std::vector<uint32_t> ks, kr;
};

struct OutMsg {
    std::vector<uint8_t> bytes;
    uint32_t v = 0;
    double block_ms = 0;
};

struct Shared {
    const pa_service_config* cfg;
    uint32_t n;
    std::atomic<bool> stop{false};
    std::atomic<int> code{0};  // first fatal exit code
    BoundedQueue<SeedMsg> seeds;
    BoundedQueue<KeyMsg> keys;
    BoundedQueue<OutMsg> outs;
    std::mutex print_mu;
    void* seed_sock = nullptr;
    void* key_sock = nullptr;
    void* out_sock = nullptr;
    Shared(const pa_service_config* c, uint32_t n_)
        : cfg(c), n(n_), seeds(c->input_blocks_to_cache), keys(c->input_blocks_to_cache),
          outs(c->output_blocks_to_cache) {}
    void fail(int rc) {
        int z = 0;
        code.compare_exchange_strong(z, rc);
        stop = true;
        seeds.close();
        keys.close();
        outs.close();
    }
    void say(const char* fmt, ...) __attribute__((format(printf, 2, 3))) {
        std::lock_guard<std::mutex> l(print_mu);
        va_list ap;
        va_start(ap, fmt);
        std::vprintf(fmt, ap);
        va_end(ap);
        std::printf("\n");
        std::fflush(stdout);
    }
};

bool read_file(const char* path, size_t need, std::vector<uint8_t>* out, int missing_rc, int short_rc, int* rc) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        *rc = missing_rc;
        return false;
    }
    f.seekg(0, std::ios::end);
    const size_t len = (size_t)f.tellg();
    f.seekg(0, std::ios::beg);
    if (len < need) {
        *rc = short_rc;
        return false;
    }
    out->resize(need);
    f.read(reinterpret_cast<char*>(out->data()), (std::streamsize)need);
    return true;
}

// Receives one frame of exactly `size` bytes; false on a size mismatch or a lost peer (the caller
// drops the rest of the message and starts over, like the reference's retry).
bool recv_exact(void* sock, void* buf, size_t size, int* more) {
    int64_t got = pa_zmq_recv(sock, buf, size, more);
    return got == (int64_t)size;
}

void drain(void* sock, int more) {
    uint8_t tmp[64];
    while (more) {
        if (pa_zmq_recv(sock, tmp, sizeof(tmp), &more) < 0) return;
    }
}

void seed_thread(Shared* sh) {
    const uint32_t n = sh->n;
    if (!sh->cfg->use_matrix_seed_server) {
        std::vector<uint8_t> bytes;
        int rc = 0;
        if (!read_file(sh->cfg->toeplitz_seed_path, n / 8, &bytes, 103, 104, &rc)) {
            sh->say("Can't use seed file \"%s\" (exit %d)", sh->cfg->toeplitz_seed_path, rc);
            sh->fail(rc);
            return;
        }
        SeedMsg m;
        m.reuse = -1;  // one seed for every block
        m.words.resize(n / 32);
        std::memcpy(m.words.data(), bytes.data(), n / 8);
        sh->seeds.push(std::move(m));
        return;
    }
    while (!sh->stop) {
        SeedMsg m;
        m.words.resize(n / 32);
        int more = 0;
        int64_t got = pa_zmq_recv(sh->seed_sock, &m.reuse, sizeof(m.reuse), &more);
        if (got < 0 && sh->stop) return;
        if (got != (int64_t)sizeof(m.reuse) || !more) {
            if (got >= 0) sh->say("Error receiving reuse_seed_amount from Seedserver! Retrying...");
            drain(sh->seed_sock, got >= 0 ? more : 0);
            continue;
        }
        if (!recv_exact(sh->seed_sock, m.words.data(), n / 8, &more)) {
            if (sh->stop) return;
            sh->say("Error receiving data from Seedserver! Retrying...");
            drain(sh->seed_sock, more);
            continue;
        }
        drain(sh->seed_sock, more);
        if (sh->cfg->show_zeromq_status) sh->say("Seed Block received");
        if (!sh->seeds.push(std::move(m))) return;
    }
}

void key_thread(Shared* sh) {
    const uint32_t n = sh->n;
    if (!sh->cfg->use_key_server) {
        std::vector<uint8_t> bytes;
        int rc = 0;
        const size_t need = ((size_t)n / 32 + 1) * 4;
        if (!read_file(sh->cfg->keyfile_path, need, &bytes, 105, 106, &rc)) {
            sh->say("Can't use key file \"%s\" (exit %d)", sh->cfg->keyfile_path, rc);
            sh->fail(rc);
            return;
        }
        const uint32_t v = sh->cfg->vertical_len;
        if (v == 0 || v >= n || (v & 31u)) {
            sh->fail(102);
            return;
        }
        KeyMsg m;
        m.v = v;
        m.flags = (sh->cfg->do_xor_key_rest ? PA_FLAG_XOR_KEY_REST : 0u) | (sh->cfg->do_compress ? PA_FLAG_COMPRESS : 0u);
        std::vector<uint32_t> recv(n / 32 + 1);
        std::memcpy(recv.data(), bytes.data(), need);
        m.ks.resize(n / 32);
        m.kr.resize(v / 32 + 1);
        pa_key_split(recv.data(), n, v, m.ks.data(), m.kr.data());
        while (!sh->stop)  // the same key every block
            if (!sh->keys.push(m)) return;
        return;
    }
    while (!sh->stop) {
        uint8_t do_xor = 0, do_compress = 0;
        uint32_t vb = 0;
        int more = 0;
        int64_t got = pa_zmq_recv(sh->key_sock, &do_xor, 1, &more);
        if (got < 0 && sh->stop) return;
        if (got != 1 || !more || !recv_exact(sh->key_sock, &do_compress, 1, &more) || !more ||
            !recv_exact(sh->key_sock, &vb, 4, &more) || !more) {
            if (sh->stop) return;
            sh->say("Error receiving key header from Keyserver! Retrying...");
            drain(sh->key_sock, got >= 0 ? more : 0);
            continue;
        }
        KeyMsg m;
        m.v = vb * 32u;
        if (m.v == 0 || m.v >= n) {
            sh->say("Invalid vertical_block %u from Keyserver! Skipping block...", vb);
            drain(sh->key_sock, more);
            continue;
        }
        const uint32_t h = n - m.v;
        m.flags = (do_xor ? PA_FLAG_XOR_KEY_REST : 0u) | (do_compress ? PA_FLAG_COMPRESS : 0u);
        m.ks.assign(n / 32, 0u);
        bool ok;
        if (do_xor) {
            std::vector<uint32_t> recv(n / 32 + 1);
            ok = recv_exact(sh->key_sock, recv.data(), recv.size() * 4, &more);
            if (ok) {
                m.kr.resize(m.v / 32 + 1);
                pa_key_split(recv.data(), n, m.v, m.ks.data(), m.kr.data());
            }
        } else {
            ok = recv_exact(sh->key_sock, m.ks.data(), ((size_t)h / 32 + 1) * 4, &more);
            if (ok) m.ks[h / 32] &= 0x80000000u;  // bits past h are not key_start
        }
        if (!ok) {
            if (sh->stop) return;
            sh->say("Error receiving key data from Keyserver! Retrying...");
            drain(sh->key_sock, more);
            continue;
        }
        drain(sh->key_sock, more);
        if (sh->cfg->show_zeromq_status) sh->say("Key Block received");
        if (!sh->keys.push(std::move(m))) return;
    }
}

bool load_expected_hash(const char* path, uint8_t out[32]) {
    std::ifstream f(path);
    if (!f) return false;
    std::string line;
    while (std::getline(f, line)) {
        size_t a = line.find_first_not_of(" \t\r");
        if (a == std::string::npos || line[a] == ';' || line[a] == '#') continue;
        std::string tok = line.substr(a, 64);
        if (tok.size() < 64) return false;
        for (int i = 0; i < 32; ++i) {
            unsigned v = 0;
            if (std::sscanf(tok.c_str() + 2 * i, "%2x", &v) != 1) return false;
            out[i] = (uint8_t)v;
        }
        return true;
    }
    return false;
}

void sender_thread(Shared* sh, int64_t max_blocks, std::atomic<int64_t>* sent) {
    const pa_service_config* c = sh->cfg;
    uint8_t expected[32] = {};
    if (c->verify_ampout && !load_expected_hash(c->ampout_sha3_path, expected)) {
        sh->say("Can't read the expected ampout hash from \"%s\"", c->ampout_sha3_path);
        sh->fail(102);
        return;
    }
    int32_t to_store = c->store_first_ampouts_in_file;
    std::ofstream store;
    if (to_store != 0) store.open(c->ampout_path, std::ios::binary);
    auto last = std::chrono::steady_clock::now();
    while (max_blocks < 0 || *sent < max_blocks) {
        OutMsg m;
        if (!sh->outs.pop(&m)) return;
        if (c->verify_ampout) {
            uint8_t got[32];
            pa_sha3_256(m.bytes.data(), std::min<size_t>(m.bytes.size(), m.v / 8), got);
            if (std::memcmp(got, expected, 32) != 0) {
                sh->say("VERIFICATION FAILED!");
                sh->fail(101);
                return;
            }
            sh->say("VERIFIED!");
        }
        if (to_store != 0 && store) {
            store.write(reinterpret_cast<const char*>(m.bytes.data()), (std::streamsize)m.bytes.size());
            store.flush();
            if (to_store > 0 && --to_store == 0) store.close();
        }
        if (c->host_ampout_server) {
            for (;;) {
                int rc = pa_zmq_send(sh->out_sock, m.bytes.data(), m.bytes.size(), 0);
                if (rc == 0) break;
                if (rc == -1 || sh->stop) return;
                sh->say("Error sending data to AMPOUT client! Retrying...");
            }
            if (c->show_zeromq_status) sh->say("Block sent to AMPOUT Client");
        }
        const auto now = std::chrono::steady_clock::now();
        const double us = std::chrono::duration<double, std::micro>(now - last).count();
        last = now;
        if (c->show_ampout >= 0) {
            sh->say("Blocktime: %.3f ms => %.1f Mbit/s (GPU %.3f ms)", us / 1000.0, sh->n / us, m.block_ms);
            for (int i = 0; i < std::min<int>(c->show_ampout, (int)m.bytes.size()); ++i)
                sh->say("0x%02X", m.bytes[i]);
        }
        ++*sent;
    }
}

}  // namespace

extern "C" int pa_service_run(const pa_service_config* cfg, int64_t max_blocks) {
    if (!cfg || cfg->factor_exp < 10 || cfg->factor_exp > 30) return 102;
    const uint32_t n = 1u << cfg->factor_exp;
    pa_engine* eng = nullptr;
    pa_config ec{cfg->gpu_device_id_to_use, n, cfg->reduction_exp, cfg->pre_mul_reduction_exp, 0.25f};
    if (pa_create(&ec, &eng) != PA_OK) return 2;
    Shared sh(cfg, n);
    int rc = 0;
    if (cfg->use_matrix_seed_server) rc |= pa_zmq_open(PA_ZMQ_PULL, cfg->address_seed_in, 0, &sh.seed_sock);
    if (cfg->use_key_server) rc |= pa_zmq_open(PA_ZMQ_PULL, cfg->address_key_in, 0, &sh.key_sock);
    if (cfg->host_ampout_server) rc |= pa_zmq_open(PA_ZMQ_PUSH, cfg->address_amp_out, 1, &sh.out_sock);
    if (rc) {
        pa_zmq_close(sh.seed_sock);
        pa_zmq_close(sh.key_sock);
        pa_zmq_close(sh.out_sock);
        pa_destroy(eng);
        return 102;
    }
    std::atomic<int64_t> sent{0};
    std::thread ts(seed_thread, &sh), tk(key_thread, &sh), to(sender_thread, &sh, max_blocks, &sent);

    int64_t done = 0;
    std::vector<uint8_t> out;
    while (!sh.stop && (max_blocks < 0 || done < max_blocks)) {
        KeyMsg k;
        if (!sh.keys.pop(&k)) break;
        out.assign(pa_output_bytes(n, k.v, k.flags), 0);
        pa_stats st{};
        int prc;
        for (;;) {
            prc = pa_process(eng, k.ks.data(), k.kr.empty() ? nullptr : k.kr.data(), n, k.v, k.flags, out.data(), &st);
            if (prc != PA_ERR_NO_SEED) break;
            SeedMsg s;  // the previous seed is used up (or none yet): take the next one
            if (!sh.seeds.pop(&s)) {
                prc = PA_ERR_NO_SEED;
                break;
            }
            if (pa_set_seed(eng, s.words.data(), n, s.reuse) != PA_OK) {
                prc = PA_ERR_CUDA;
                break;
            }
        }
        if (prc != PA_OK) {
            if (!sh.stop) {
                sh.say("Block failed: %s", pa_error_string(prc));
                sh.fail(2);
            }
            break;
        }
        OutMsg m;
        m.bytes = out;
        m.v = k.v;
        m.block_ms = st.gpu_ms;
        if (!sh.outs.push(std::move(m))) break;
        ++done;
    }
    to.join();  // the sender finishes the handed-off blocks (or stops on an error)
    sh.stop = true;
    sh.seeds.close();
    sh.keys.close();
    sh.outs.close();
    if (sh.seed_sock) pa_zmtp_interrupt(sh.seed_sock);
    if (sh.key_sock) pa_zmtp_interrupt(sh.key_sock);
    ts.join();
    tk.join();
    pa_zmq_close(sh.seed_sock);
    pa_zmq_close(sh.key_sock);
    pa_zmq_close(sh.out_sock);
    pa_destroy(eng);
    return sh.code.load();
}
