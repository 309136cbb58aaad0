#!/bin/sh
# Builds oracle/_ref/ref_driver, the reference's own CPU-only build (test
# infrastructure: it pins the oracle and makes the golden fixtures), from the
# reference source tree where it lies. REFERENCE overrides the location; the
# default is where the build container mounts the tree read-only. When the
# tree is absent (as on the GPU machines), the Makefile skips the target.
REFERENCE="${REFERENCE:-/root/reference}"
exec make -s -C "$(dirname "$0")" ref REFERENCE="$REFERENCE"
