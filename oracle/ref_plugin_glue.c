/*
 * Test glue for the GPU model plugin (charm_3d_gb300/csrc/plugin/charm_model_gpu.c)
 * inside the reference build: flatten ref_driver.c's current forest through the
 * plugin, build the plugin's configuration from ref_driver.c's context, and
 * swap the plugin pair into that context so that ref_run (the loop of
 * charm_timesteps) steps through it on the GPU.  Oracle-side test
 * infrastructure; only the steps after ref_plugin_use_gpu and
 * ref_plugin_finish reach the GPU.
 */
#include "charm_globals.h"
#include "charm_gpu.h"

int charm_model_gpu_flatten(p4est_t *p4est, charm_gpu_mesh_t *mesh);
int charm_model_gpu_flatten_hex(charm_gpu_mesh_t *mesh, charm_gpu_hex_t *hex);
int charm_model_gpu_config(charm_ctx_t *ctx, int precision, charm_gpu_config_t *cfg);
void charm_model_gpu_init(charm_ctx_t *ctx, int precision, int device);
void charm_model_gpu_finalize(p4est_t *p4est);
int charm_model_gpu_status(void);
p4est_t *ref_driver_p4est(void);

/* Register the plugin's timestep_single_fn / get_dt_fn in the current
 * context, as a reference main would after charm_init_context_yaml. */
int ref_plugin_use_gpu(int precision)
{
    charm_model_gpu_init(charm_get_ctx(ref_driver_p4est()), precision, 0);
    return 0;
}

/* Bring the plugin's newest state back into the quadrants and release its
 * handle; returns the plugin's status (0, or the first failing CHARM_GPU_*). */
int ref_plugin_finish(void)
{
    const int st = charm_model_gpu_status();
    charm_model_gpu_finalize(ref_driver_p4est());
    return st;
}

int ref_plugin_flatten(charm_gpu_mesh_t *out) { return charm_model_gpu_flatten(ref_driver_p4est(), out); }

/* the general-hexahedron form: returns 1 when the plugin would upload it
 * (-1 on a flattening error) */
int ref_plugin_flatten_hex(charm_gpu_mesh_t *out, charm_gpu_hex_t *hex)
{
    int rc = charm_model_gpu_flatten(ref_driver_p4est(), out);
    if (rc) return -1;
    return charm_model_gpu_flatten_hex(out, hex);
}

int ref_plugin_config(int precision, charm_gpu_config_t *out)
{
    return charm_model_gpu_config(charm_get_ctx(ref_driver_p4est()), precision, out);
}
