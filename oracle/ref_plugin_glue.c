/*
 * Test glue for the GPU model plugin (charm_3d_gb300/csrc/plugin/charm_model_gpu.c)
 * inside the reference build: flatten ref_driver.c's current forest through the
 * plugin and build the plugin's configuration from ref_driver.c's context.
 * Oracle-side test infrastructure; no GPU calls.
 */
#include "charm_globals.h"
#include "charm_gpu.h"

int charm_model_gpu_flatten(p4est_t *p4est, charm_gpu_mesh_t *mesh);
int charm_model_gpu_flatten_hex(charm_gpu_mesh_t *mesh, charm_gpu_hex_t *hex);
int charm_model_gpu_config(charm_ctx_t *ctx, int precision, charm_gpu_config_t *cfg);
p4est_t *ref_driver_p4est(void);

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
