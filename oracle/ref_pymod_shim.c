/*
 * Python 3 module-init shim for the reference's Python-2 C extensions
 * (test infrastructure only; used by oracle/build_ref.py).
 *
 * The reference sources are compiled where they lie: this file #includes
 * one of them (REF_SRC) unchanged.  Their Py2 init function calls
 * Py_InitModule3(name, methods, doc); the macro below only records the
 * method table, and SHIM_INIT wraps it in a Py3 PyModuleDef.
 */
#include <Python.h>

static PyMethodDef *shim_methods_;
#define Py_InitModule3(name, methods, doc) (shim_methods_ = (methods), (PyObject *)NULL)
/* Python 3 has one integer type */
#define PyInt_AsLong PyLong_AsLong
/* Python 2's PyList_Check expanded to a parenthesised expression, and some
 * sources use it bare (`else if PyList_Check(x)`) */
#undef PyList_Check
#define PyList_Check(op) (PyType_FastSubclass(Py_TYPE(op), Py_TPFLAGS_LIST_SUBCLASS))

#include REF_SRC

static struct PyModuleDef shim_def_ = {PyModuleDef_HEAD_INIT, SHIM_NAME, NULL, -1, NULL};

PyMODINIT_FUNC SHIM_INIT(void)
{
    SHIM_OLD_INIT();
    if (PyErr_Occurred()) return NULL;
    shim_def_.m_methods = shim_methods_;
    return PyModule_Create(&shim_def_);
}
