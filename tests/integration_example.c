/* The C usage example shown in the integration guide: build one tetrahedral body, step it 120
 * times through the C ABI and read its state back. tests/test_abi.py compiles it with
 * -Wall -Werror against include/b3g.h and links it against libb3g.so. */
#include <stdint.h>
#include <stdio.h>

#include "b3g.h"

void example(uint32_t n, float* xyz, float* vel, const int32_t* types, const float* damp, uint32_t T,
             const uint32_t* ids, const float* E, const float* nu, const float* rho)
{
	b3g_context* ctx; b3g_context_create(0, &ctx);
	b3g_body_desc d = {0};
	d.vertex_count = n; d.positions = xyz; d.types = types; d.damping = damp;
	d.tet_count = T; d.tets = ids; d.tet_young = E; d.tet_poisson = nu; d.tet_density = rho;
	d.gravity[1] = -9.8f;
	b3g_body* body; if (b3g_body_create(ctx, &d, &body) != B3G_OK) puts(b3g_last_error());
	b3g_solver_config cfg; b3g_solver_config_default(&cfg);
	cfg.max_pcg_iterations = 200; cfg.pcg_tolerance = 1e-5;
	b3g_step_stats st;
	for (int s = 0; s < 120; ++s) b3g_body_step(body, 1.0f / 60, &cfg, &st);
	b3g_body_get_state(body, xyz, vel);
	b3g_body_destroy(body); b3g_context_destroy(ctx);
}
