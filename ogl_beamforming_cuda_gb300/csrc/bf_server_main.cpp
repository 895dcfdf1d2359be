/*
 * bf_server_main.cpp -- ogl_beamformer_server: serves the reference's
 * shared-memory client protocol ("/ogl_beamformer_shared_memory", version 11)
 * on this library until SIGINT or SIGTERM.
 *
 * Usage: ogl_beamformer_server [--idle-exit-ms N] [--das-precision P]
 *   --idle-exit-ms N    exit after N ms without work
 *   --das-precision P   HERCULES DAS arithmetic: 0 FP32 (default), 1 FP16 table
 */
#include "ogl_beamformer_lib.h"

#include <csignal>
#include <cstdio>
#include <cstdlib>
#include <cstring>

static void on_signal(int) { beamformer_gb300_serve_stop(); }

int main(int argc, char **argv)
{
	int32_t idle = -1;
	for (int i = 1; i < argc; i++) {
		if (!std::strcmp(argv[i], "--idle-exit-ms") && i + 1 < argc) {
			idle = std::atoi(argv[++i]);
		} else if (!std::strcmp(argv[i], "--das-precision") && i + 1 < argc) {
			if (!beamformer_gb300_set_das_precision(std::atoi(argv[++i]))) {
				std::fprintf(stderr, "ogl_beamformer_server: %s\n", beamformer_get_last_error_string());
				return 2;
			}
		} else {
			std::fprintf(stderr, "usage: ogl_beamformer_server [--idle-exit-ms N] [--das-precision P]\n");
			return 2;
		}
	}
	std::signal(SIGINT, on_signal);
	std::signal(SIGTERM, on_signal);
	std::fprintf(stderr, "ogl_beamformer_server: serving /ogl_beamformer_shared_memory (version %u)\n",
	             BEAMFORMER_SHARED_MEMORY_VERSION);
	const int32_t r = beamformer_gb300_serve(idle);
	beamformer_gb300_shutdown();
	return r == 0 ? 0 : 1;
}
