/*
 * TEST-ONLY stand-ins for the two POY / OCaml runtime functions that
 * integration/poy_stubs.c calls outside libpoyalgn.so (seq_prepend from
 * POY's seq.c, caml_failwith from the OCaml runtime), so that the stub file
 * links into a shared library with no undefined symbol left. Nothing here
 * runs an alignment.
 */
#include <assert.h>
#include <stdio.h>
#include <stdlib.h>

#include "seq.h"

void seq_prepend(seqt a, SEQT v)
{
    a->begin--;
    *a->begin = v;
    a->len++;
}

void caml_failwith(const char *msg)
{
    fprintf(stderr, "failwith: %s\n", msg);
    abort();
}
