// ref_cec_wrap.cc -- extern "C" access to the reference's own CPU objective.
//
// TEST INFRASTRUCTURE ONLY. Compiled together with the reference's CEC2014.cc (in place,
// from the reference tree) into oracle/_ref/libref_cec.so by `make -C oracle ref`; used to
// pin this project's objective restatement and to make golden vectors. CEC2014::Initilize
// (CUDA_EA_library/CEC2014.cc:290-420) reads input_data/M_<f>_D<d>.txt and
// input_data/shift_data_<f>.txt relative to the working directory, so ref_cec_init changes
// into `data_dir` for the duration of that call.
#include "CEC2014.h"

#include <unistd.h>

#include <climits>

static CEC2014 *g_cec = nullptr;

extern "C" int ref_cec_init(int func_id, int dim, const char *data_dir)
{
    char cwd[PATH_MAX];
    if (!getcwd(cwd, sizeof cwd)) return -1;
    if (chdir(data_dir) != 0) return -2;
    if (g_cec) { g_cec->Unitilize(); delete g_cec; }
    g_cec = new CEC2014();
    g_cec->Initilize(func_id, dim);
    if (chdir(cwd) != 0) return -3;
    return 0;
}

// CEC2014::EvaluateFitness(double*) (CEC2014.cc:13-145): returns f(x) - f*.
extern "C" double ref_cec_eval(const double *x)
{
    return g_cec->EvaluateFitness(const_cast<double *>(x));
}

extern "C" void ref_cec_eval_batch(const double *x, int n, int ld, double *out)
{
    for (int i = 0; i < n; ++i) out[i] = g_cec->EvaluateFitness(const_cast<double *>(x + (size_t)i * ld));
}

extern "C" void ref_cec_free(void)
{
    if (g_cec) { g_cec->Unitilize(); delete g_cec; g_cec = nullptr; }
}
