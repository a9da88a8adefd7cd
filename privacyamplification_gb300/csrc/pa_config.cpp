// pa_config.cpp -- config.yaml surface of the host loop (readConfig, PrivacyAmplification.cu:1228-1272).
// The reference's config is a flat list of `key: value` scalars; this reader handles exactly that:
// comments (#), single/double quotes, integers and true/false (also yes/no, on/off).
#include "../../include/pa_service.h"

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>

namespace {

void set_str(char* dst, size_t cap, const std::string& v) {
    std::snprintf(dst, cap, "%s", v.c_str());
}

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

// Value text after the colon: strips a trailing comment outside quotes and the quotes themselves.
std::string scalar(const std::string& raw) {
    std::string v = trim(raw);
    if (!v.empty() && (v[0] == '\'' || v[0] == '"')) {
        const char q = v[0];
        std::string out;
        for (size_t i = 1; i < v.size(); ++i) {
            if (v[i] == q) {
                if (q == '\'' && i + 1 < v.size() && v[i + 1] == '\'') {  // '' inside single quotes
                    out += '\'';
                    ++i;
                    continue;
                }
                return out;
            }
            out += v[i];
        }
        return out;
    }
    size_t hash = v.find(" #");
    if (v.rfind('#', 0) == 0) return std::string();
    if (hash != std::string::npos) v = v.substr(0, hash);
    return trim(v);
}

bool as_bool(const std::string& v, int32_t* out) {
    std::string l;
    for (char c : v) l += (char)std::tolower((unsigned char)c);
    if (l == "true" || l == "yes" || l == "on" || l == "1") { *out = 1; return true; }
    if (l == "false" || l == "no" || l == "off" || l == "0") { *out = 0; return true; }
    return false;
}

template <class T>
bool as_int(const std::string& v, T* out) {
    if (v.empty()) return false;
    char* end = nullptr;
    long long x = std::strtoll(v.c_str(), &end, 0);
    if (!end || *end) {
        int32_t b;  // the reference reads `true` for an integer key as 1 (store_first_ampouts_in_file)
        if (as_bool(v, &b)) { *out = (T)b; return true; }
        return false;
    }
    *out = (T)x;
    return true;
}

}  // namespace

extern "C" void pa_service_config_default(pa_service_config* c) {
    std::memset(c, 0, sizeof(*c));
    c->factor_exp = 27;
    c->reuse_seed_amount = 0;
    c->vertical_len = 50331648u;
    c->do_xor_key_rest = 1;
    c->do_compress = 1;
    c->reduction_exp = 11;
    c->pre_mul_reduction_exp = 5;
    c->gpu_device_id_to_use = 0;
    c->input_blocks_to_cache = 16;
    c->output_blocks_to_cache = 16;
    c->show_ampout = 0;
    c->show_zeromq_status = 1;
    c->use_matrix_seed_server = 1;
    set_str(c->address_seed_in, sizeof(c->address_seed_in), "tcp://127.0.0.1:45555");
    set_str(c->toeplitz_seed_path, sizeof(c->toeplitz_seed_path), "toeplitz_seed.bin");
    c->use_key_server = 1;
    set_str(c->address_key_in, sizeof(c->address_key_in), "tcp://127.0.0.1:47777");
    set_str(c->keyfile_path, sizeof(c->keyfile_path), "keyfile.bin");
    c->host_ampout_server = 1;
    set_str(c->address_amp_out, sizeof(c->address_amp_out), "tcp://127.0.0.1:48888");
    c->store_first_ampouts_in_file = 1;
    c->verify_ampout = 1;
    c->verify_ampout_threads = 8;
    set_str(c->ampout_sha3_path, sizeof(c->ampout_sha3_path), "ampout.sh3");
    set_str(c->ampout_path, sizeof(c->ampout_path), "ampout.bin");
}

extern "C" int pa_service_config_load(const char* path, pa_service_config* c) {
    if (!path || !c) return 102;
    std::ifstream f(path);
    if (!f) return 102;
    std::string line;
    while (std::getline(f, line)) {
        std::string t = trim(line);
        if (t.empty() || t[0] == '#' || t == "---") continue;
        size_t colon = t.find(':');
        if (colon == std::string::npos) continue;
        const std::string key = trim(t.substr(0, colon));
        const std::string v = scalar(t.substr(colon + 1));
        int32_t b;
        if (key == "factor_exp") as_int(v, &c->factor_exp);
        else if (key == "reuse_seed_amount") as_int(v, &c->reuse_seed_amount);
        else if (key == "vertical_len") as_int(v, &c->vertical_len);
        else if (key == "do_xor_key_rest") { if (as_bool(v, &b)) c->do_xor_key_rest = b; }
        else if (key == "do_compress") { if (as_bool(v, &b)) c->do_compress = b; }
        else if (key == "reduction_exp") as_int(v, &c->reduction_exp);
        else if (key == "pre_mul_reduction_exp") as_int(v, &c->pre_mul_reduction_exp);
        else if (key == "gpu_device_id_to_use") as_int(v, &c->gpu_device_id_to_use);
        else if (key == "input_blocks_to_cache") as_int(v, &c->input_blocks_to_cache);
        else if (key == "output_blocks_to_cache") as_int(v, &c->output_blocks_to_cache);
        else if (key == "show_ampout") as_int(v, &c->show_ampout);
        else if (key == "show_zeromq_status") { if (as_bool(v, &b)) c->show_zeromq_status = b; }
        else if (key == "use_matrix_seed_server") { if (as_bool(v, &b)) c->use_matrix_seed_server = b; }
        else if (key == "address_seed_in") set_str(c->address_seed_in, sizeof(c->address_seed_in), v);
        else if (key == "toeplitz_seed_path") set_str(c->toeplitz_seed_path, sizeof(c->toeplitz_seed_path), v);
        else if (key == "use_key_server") { if (as_bool(v, &b)) c->use_key_server = b; }
        else if (key == "address_key_in") set_str(c->address_key_in, sizeof(c->address_key_in), v);
        else if (key == "keyfile_path") set_str(c->keyfile_path, sizeof(c->keyfile_path), v);
        else if (key == "host_ampout_server") { if (as_bool(v, &b)) c->host_ampout_server = b; }
        else if (key == "address_amp_out") set_str(c->address_amp_out, sizeof(c->address_amp_out), v);
        else if (key == "store_first_ampouts_in_file") as_int(v, &c->store_first_ampouts_in_file);
        else if (key == "verify_ampout") { if (as_bool(v, &b)) c->verify_ampout = b; }
        else if (key == "verify_ampout_threads") as_int(v, &c->verify_ampout_threads);
        else if (key == "ampout_sha3_path") set_str(c->ampout_sha3_path, sizeof(c->ampout_sha3_path), v);
        else if (key == "ampout_path") set_str(c->ampout_path, sizeof(c->ampout_path), v);
    }
    return 0;
}
