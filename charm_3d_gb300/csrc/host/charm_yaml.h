/*
 * charm_yaml.h - reader of the YAML subset used by CHARM_3D's case files
 * (task.yaml), into a tree of maps, sequences and scalars.  See charm_yaml.c
 * for what is and is not supported.
 */
#ifndef CHARM_YAML_H
#define CHARM_YAML_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { CHARM_Y_SCALAR = 0, CHARM_Y_MAP = 1, CHARM_Y_SEQ = 2 };

typedef struct charm_ynode {
    int type;
    char *str;                     /* scalar text (quotes removed) */
    int n, cap;                    /* entries of a map or sequence */
    char **keys;                   /* map keys (NULL entries in a sequence) */
    struct charm_ynode **items;
} charm_ynode_t;

/* Parse text / a file; NULL on error with the message (and line) in err. */
charm_ynode_t *charm_yaml_parse(const char *text, char *err, size_t errlen);
charm_ynode_t *charm_yaml_load(const char *path, char *err, size_t errlen);
void charm_yaml_free(charm_ynode_t *n);

/* Lookups: the value of key in a map (NULL if absent or not a map); scalar
 * conversions return 0 on success, -1 if the node is missing or not a
 * number of that kind. */
const charm_ynode_t *charm_yaml_get(const charm_ynode_t *map, const char *key);
int charm_yaml_double(const charm_ynode_t *n, double *out);
int charm_yaml_int(const charm_ynode_t *n, int *out);
const char *charm_yaml_str(const charm_ynode_t *n);

#ifdef __cplusplus
}
#endif

#endif
