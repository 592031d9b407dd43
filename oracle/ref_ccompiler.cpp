/* Test infrastructure only: builds the reference's pysiml/_ccompiler.cpp as a
 * Python-3 module "_ccompiler" (SMILEStoMatrices). */
#include "ref_compat.h"
#include "_ccompiler.cpp"

static struct PyModuleDef siml_ref_ccompiler_def = {
    PyModuleDef_HEAD_INIT, "_ccompiler", NULL, -1, _ccompiler_methods,
    NULL, NULL, NULL, NULL};

extern "C" PyMODINIT_FUNC PyInit__ccompiler(void) {
    PyObject* m = PyModule_Create(&siml_ref_ccompiler_def);
    if (m == NULL) return NULL;
    if (_import_array() < 0) return NULL;
    return m;
}
