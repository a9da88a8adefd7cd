/* pa_service.h -- the host loop around the engine: config.yaml surface, ZeroMQ-wire key/seed ingest and
 * ampout egress, SHA3-256 output check.
 *
 * Replaces the reference's main() and its three I/O threads (PrivacyAmplification.cu:1394-1680,
 * 969-1225) and readConfig() (PrivacyAmplification.cu:1228-1272).  libzmq is not a dependency: the
 * sockets below speak ZMTP 3.0 (NULL mechanism, PUSH/PULL) over TCP themselves, one peer per socket.
 *
 * Exit codes (returned, never exit()): 0 done, 101 ampout verification failed, 102 config unreadable,
 * 103/104 seed file missing/too short, 105/106 key file missing/too short, 2 engine error. */
#ifndef PA_SERVICE_H
#define PA_SERVICE_H

#include "pa_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Keys and defaults of the reference's config.yaml (PrivacyAmplification.cu:1243-1271). */
typedef struct pa_service_config {
    uint32_t factor_exp;            /* sample_size n = 2^factor_exp (27) */
    int32_t reuse_seed_amount;      /* file seed: 0 */
    uint32_t vertical_len;          /* file key: v (50331648) */
    int32_t do_xor_key_rest;        /* file key: 1 */
    int32_t do_compress;            /* file key: 1 */
    uint32_t reduction_exp;         /* 11, accepted for compatibility */
    uint32_t pre_mul_reduction_exp; /* 5, accepted for compatibility */
    int32_t gpu_device_id_to_use;   /* 0 */
    uint32_t input_blocks_to_cache; /* queue depth of received seeds / keys (16) */
    uint32_t output_blocks_to_cache;/* queue depth of results waiting to be sent (16) */
    int32_t show_ampout;            /* < 0 quiet; >= 0 block time; > 0 also this many output bytes (0) */
    int32_t show_zeromq_status;     /* 1 */
    int32_t use_matrix_seed_server; /* 1: seeds from address_seed_in, else from toeplitz_seed_path */
    char address_seed_in[256];      /* tcp://127.0.0.1:45555 */
    char toeplitz_seed_path[1024];  /* toeplitz_seed.bin */
    int32_t use_key_server;         /* 1: keys from address_key_in, else from keyfile_path */
    char address_key_in[256];       /* tcp://127.0.0.1:47777 */
    char keyfile_path[1024];        /* keyfile.bin */
    int32_t host_ampout_server;     /* 1: results to address_amp_out (bound here) */
    char address_amp_out[256];      /* tcp://127.0.0.1:48888 */
    int32_t store_first_ampouts_in_file; /* write the first k results to ampout.bin (-1 all) (1) */
    int32_t verify_ampout;          /* 1: SHA3-256 of every result's v/8 bytes must equal the expected hash */
    uint32_t verify_ampout_threads; /* 8, accepted for compatibility (verification runs on the sender) */
    char ampout_sha3_path[1024];    /* expected hash: "<64 hex digits> ..." line, ';' comments (ampout.sh3) */
    char ampout_path[1024];         /* where store_first_ampouts_in_file writes (ampout.bin) */
} pa_service_config;

PA_API void pa_service_config_default(pa_service_config* cfg);
/* Reads `key: value` lines (quotes, comments, true/false) over the defaults; unknown keys are ignored.
 * Returns 0, or 102 when the file cannot be read. */
PA_API int pa_service_config_load(const char* path, pa_service_config* cfg);
/* Runs the loop: blocks are hashed in arrival order with the reference's seed-reuse rule.  Stops after
 * max_blocks results have been handed off (and sent, when host_ampout_server), or never when < 0. */
PA_API int pa_service_run(const pa_service_config* cfg, int64_t max_blocks);

/* SHA3-256 (FIPS 202), the reference's isSha3 check (PrivacyAmplification.cu:1120-1128). */
PA_API void pa_sha3_256(const void* data, size_t len, uint8_t out[32]);

/* ZMTP 3.0 sockets.  type: PA_ZMQ_PULL or PA_ZMQ_PUSH; endpoint "tcp://host:port"; bind = 1 listens
 * and serves one peer at a time, bind = 0 connects (retrying until the peer is up).  Handshake and
 * reconnects happen inside send/recv.  recv returns the frame size (frames larger than cap are
 * truncated and reported with their full size) and sets *more for multi-part messages; negative on
 * error or after pa_zmq_close. */
#define PA_ZMQ_PULL 7
#define PA_ZMQ_PUSH 8
PA_API int pa_zmq_open(int type, const char* endpoint, int bind, void** sock);
PA_API int64_t pa_zmq_recv(void* sock, void* buf, size_t cap, int* more);
PA_API int pa_zmq_send(void* sock, const void* buf, size_t len, int more);
PA_API void pa_zmq_close(void* sock);

#ifdef __cplusplus
}
#endif
#endif /* PA_SERVICE_H */
