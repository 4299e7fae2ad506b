// Batched stepping of many independent bodies (b3g_step_batch).
#include "api_internal.h"

#include <vector>

using namespace b3g;

struct BatchCache
{
};

void destroy_batch_cache(b3g_context* c)
{
	delete c->batch;
	c->batch = nullptr;
}

void forget_body_in_batch_cache(b3g_context* c, b3g_body* b)
{
	(void)b;
	destroy_batch_cache(c);
}

extern "C" int b3g_step_batch(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, float dt,
                              const b3g_solver_config* cfg, uint32_t steps, b3g_step_stats* stats)
{
	if (!ctx || (!bodies && count)) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	for (uint32_t s = 0; s < steps; ++s)
		for (uint32_t k = 0; k < count; ++k)
		{
			int rc = b3g_body_step(bodies[k], dt, cfg, (stats && s + 1 == steps) ? stats + k : nullptr);
			if (rc != B3G_OK) return rc;
		}
	return B3G_OK;
}
