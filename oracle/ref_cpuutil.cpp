/* Test infrastructure only: builds the reference's pysiml/_cpuutil.cpp as a
 * Python-3 module "_cpuutil" (rowHistogram101). */
#include "ref_compat.h"
#include "_cpuutil.cpp"

static struct PyModuleDef siml_ref_cpuutil_def = {
    PyModuleDef_HEAD_INIT, "_cpuutil", NULL, -1, _cpuutil_methods,
    NULL, NULL, NULL, NULL};

extern "C" PyMODINIT_FUNC PyInit__cpuutil(void) {
    PyObject* m = PyModule_Create(&siml_ref_cpuutil_def);
    if (m == NULL) return NULL;
    if (_import_array() < 0) return NULL;
    return m;
}
