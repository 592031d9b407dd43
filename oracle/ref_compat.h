/*
 * Test infrastructure only: a compatibility header that lets the reference's own
 * Python-2 C extensions (pysiml/_CPULingo.c, pysiml/_ccompiler.cpp,
 * pysiml/_cpuutil.cpp) compile unmodified as Python-3 extension modules.
 *
 * The reference sources are #included from where they lie (the include path is
 * set by oracle/Makefile); nothing of them is copied. Each ref_*.c(pp) file then
 * adds a PyInit_<name> that wraps the reference's static method table.
 */
#ifndef SIML_REF_COMPAT_H
#define SIML_REF_COMPAT_H

#include <Python.h>
#include <numpy/arrayobject.h>

/* Python 2 names used by the reference */
#define PyString_AsStringAndSize PyBytes_AsStringAndSize
#define DL_EXPORT(rtype) rtype
#define Py_InitModule3(name, methods, doc) ((void)0)

/* numpy 1.x flag name used by the reference */
#ifndef NPY_CARRAY
#define NPY_CARRAY NPY_ARRAY_CARRAY
#endif

/* The reference's init<name>() functions call import_array() from a void
 * function; the real macro returns NULL there.  Our PyInit_<name> calls
 * _import_array() itself, so the reference's call becomes a no-op. */
#undef import_array
#define import_array() ((void)0)

#endif
