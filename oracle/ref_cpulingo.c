/* Test infrastructure only: builds the reference's pysiml/_CPULingo.c as a
 * Python-3 module "_CPULingo" (multisetTanimoto3_mags, getTanimotoBlock[Parallel]). */
#include "ref_compat.h"
#include "_CPULingo.c"

static struct PyModuleDef siml_ref_cpulingo_def = {
    PyModuleDef_HEAD_INIT, "_CPULingo", NULL, -1, _CPULingo_methods,
    NULL, NULL, NULL, NULL};

PyMODINIT_FUNC PyInit__CPULingo(void) {
    PyObject* m = PyModule_Create(&siml_ref_cpulingo_def);
    if (m == NULL) return NULL;
    if (_import_array() < 0) return NULL;
    return m;
}
