/*
 * The four slu_* entry points of tools/superlu.h implemented by embedding
 * CPython and calling scipy's SuperLU (scipy.sparse.linalg.spilu, SuperLU
 * 5.x vendored by scipy) with the reference's ILU options
 * (tools/superlu.c:218-230): drop rule BASIC, drop tolerance 1e-6, fill
 * factor 2.0, NATURAL column order, no equilibration, no row permutation,
 * diagonal pivot threshold 0, SILU.  As in tools/superlu.c:142-152 the CSR
 * arrays of the preconditioner matrix are read as CSC, so SuperLU factors
 * its transpose; solves use SuperLU's own triangular solves (FACTORED).
 * Oracle build only (x86 container, Python 3 with scipy).
 */
#define PY_SSIZE_T_CLEAN
#include <Python.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "superlu.h"

typedef struct { int n, nnz; void *Ax; int *Ai, *Ap; } ccs_t;

static PyObject *g_mod = NULL;

static const char *g_src =
    "import numpy as np, scipy.sparse as sp, scipy.sparse.linalg as spla\n"
    "def factor(n, nnz, ax, ai, ap):\n"
    "    A = sp.csc_matrix((np.frombuffer(ax, np.complex128).copy(), np.frombuffer(ai, np.int32).copy(),\n"
    "                       np.frombuffer(ap, np.int32).copy()), shape=(n, n))\n"
    "    return spla.spilu(A, drop_tol=1e-6, fill_factor=2.0, drop_rule='basic', permc_spec='NATURAL',\n"
    "                      diag_pivot_thresh=0.0, options=dict(Equil=False, RowPerm='NOROWPERM', ILU_MILU='SILU'))\n"
    "def nnz(lu):\n"
    "    return (lu.L.nnz, lu.U.nnz)\n"
    "def solve(lu, b):\n"
    "    return lu.solve(np.frombuffer(b, np.complex128)).astype(np.complex128).tobytes()\n";

static void die_py(const char *what)
{
    fprintf(stderr, "slu_embed: %s failed\n", what);
    if (PyErr_Occurred()) PyErr_Print();
    exit(1);
}

static void ensure_python(void)
{
    if (g_mod) return;
    Py_Initialize();
    PyObject *code = Py_CompileString(g_src, "slu_embed", Py_file_input);
    if (!code) die_py("compile");
    g_mod = PyImport_ExecCodeModule("slu_embed", code);
    Py_DECREF(code);
    if (!g_mod) die_py("import numpy/scipy");
}

slu_matrix_t slu_create_matrix(int nrows, int ncols, int nnz, void *Ax, int *Ai, int *Ap)
{
    slu_matrix_t ret;
    ccs_t *m = malloc(sizeof(ccs_t));
    (void)ncols;
    m->n = nrows; m->nnz = nnz; m->Ax = Ax; m->Ai = Ai; m->Ap = Ap;
    ret.ptr = m;
    return ret;
}

slu_LU_t slu_compute_ilu(slu_matrix_t A)
{
    slu_LU_t ret;
    memset(&ret, 0, sizeof(ret));
    ccs_t *m = (ccs_t *)A.ptr;
    ensure_python();
    PyObject *f = PyObject_GetAttrString(g_mod, "factor");
    PyObject *args = Py_BuildValue("(iiy#y#y#)", m->n, m->nnz,
                                   (const char *)m->Ax, (Py_ssize_t)m->nnz * 16,
                                   (const char *)m->Ai, (Py_ssize_t)m->nnz * 4,
                                   (const char *)m->Ap, (Py_ssize_t)(m->n + 1) * 4);
    PyObject *lu = PyObject_CallObject(f, args);
    Py_DECREF(args); Py_DECREF(f);
    if (!lu) die_py("spilu");
    PyObject *fn = PyObject_GetAttrString(g_mod, "nnz");
    PyObject *nz = PyObject_CallFunctionObjArgs(fn, lu, NULL);
    long ln = 0, un = 0;
    if (nz && PyArg_ParseTuple(nz, "ll", &ln, &un)) {
        printf("SuperLU L dimension %dx%d; # nonzeros %ld\n", m->n, m->n, ln);
        printf("SuperLU U dimension %dx%d; # nonzeros %ld\n", m->n, m->n, un);
        fflush(stdout);
    }
    Py_XDECREF(nz); Py_DECREF(fn);
    ret.A = m;
    ret.L = lu;          /* keeps the scipy SuperLU object */
    return ret;
}

void slu_lu_solve(slu_LU_t *lu, doublecomplex *rhs, doublecomplex *x)
{
    ccs_t *m = (ccs_t *)lu->A;
    PyObject *f = PyObject_GetAttrString(g_mod, "solve");
    PyObject *b = PyBytes_FromStringAndSize((const char *)rhs, (Py_ssize_t)m->n * 16);
    PyObject *res = PyObject_CallFunctionObjArgs(f, (PyObject *)lu->L, b, NULL);
    Py_DECREF(b); Py_DECREF(f);
    if (!res) die_py("solve");
    memcpy(x, PyBytes_AsString(res), (size_t)m->n * 16);
    Py_DECREF(res);
}

void slu_LU2coo(const SuperMatrix *L, const SuperMatrix *U,
                int_t **LAi_out, int_t **LAj_out, doublecomplex **LAx_out, int_t *Lnnz,
                int_t **UAi_out, int_t **UAj_out, doublecomplex **UAx_out, int_t *Unnz)
{
    (void)L; (void)U; (void)LAi_out; (void)LAj_out; (void)LAx_out; (void)Lnnz;
    (void)UAi_out; (void)UAj_out; (void)UAx_out; (void)Unnz;
    fprintf(stderr, "slu_LU2coo is only used by the GPU build\n");
    exit(1);
}
