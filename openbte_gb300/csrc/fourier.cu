// placeholder, replaced below
#include "internal.h"
extern "C" obte_status obte_fourier_plan_create(obte_context, const obte_fourier_problem*, obte_fourier_plan*) { return OBTE_ERR_UNSUPPORTED; }
extern "C" obte_status obte_fourier_plan_destroy(obte_fourier_plan) { return OBTE_OK; }
extern "C" obte_status obte_fourier_solve(obte_fourier_plan, const obte_fourier_opts*, double*, double*, obte_fourier_info*) { return OBTE_ERR_UNSUPPORTED; }
