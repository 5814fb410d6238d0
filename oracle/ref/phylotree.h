/*
 * Found by tree/phylokernelnew.h's `#include "phylotree.h"` when the kernel
 * header is built from a staged copy that lacks tree/phylotree.h. refenv.h
 * defines PHYLOTREE_H before that include, so the real header would be empty
 * here as well: the kernels compile against the stand-ins of refenv.h.
 */
