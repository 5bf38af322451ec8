// nsm_prog.cuh — evaluation of custom propensity programs (SP_OP_* in
// include/spgpu.h): the reaction's propensity_function as postfix code,
// computed in double and rounded to float by the caller.  The host checks
// every program before upload (operands in range, stack depth at most
// SP_PROG_MAX_STACK, END reached), so the loop ends at END.
#pragma once
#include <cstdint>

#include "../../include/spgpu.h"

namespace spg {

// xs(s): the count of species s at this voxel (a register shuffle in the
// warp kernels, an array read elsewhere); v: the voxel (data functions)
template <typename XF>
__device__ __forceinline__ double run_program(const int32_t* code, const double* consts,
                                              const double* data, int n_vox, int v, XF xs,
                                              double vol, double t, int type) {
    double st[SP_PROG_MAX_STACK];
    int sp = 0;
    for (int pc = 0;;) {
        const int op = code[pc];
        switch (op) {
            case SP_OP_END: return st[sp - 1];
            case SP_OP_CONST: st[sp++] = consts[code[pc + 1]]; pc += 2; break;
            case SP_OP_X: st[sp++] = (double)xs(code[pc + 1]); pc += 2; break;
            case SP_OP_VOL: st[sp++] = vol; pc++; break;
            case SP_OP_T: st[sp++] = t; pc++; break;
            case SP_OP_TYPE: st[sp++] = (double)type; pc++; break;
            case SP_OP_DATA: st[sp++] = data[(size_t)code[pc + 1] * n_vox + v]; pc += 2; break;
            case SP_OP_NEG: st[sp - 1] = -st[sp - 1]; pc++; break;
            case SP_OP_NOT: st[sp - 1] = st[sp - 1] == 0.0 ? 1.0 : 0.0; pc++; break;
            case SP_OP_POWI: {
                const int n = code[pc + 1];
                const int m = n < 0 ? -n : n;
                double r = 1.0;
                for (int q = 0; q < m; q++) r = r * st[sp - 1];
                st[sp - 1] = n < 0 ? 1.0 / r : r;
                pc += 2;
                break;
            }
            case SP_OP_EXP: st[sp - 1] = exp(st[sp - 1]); pc++; break;
            case SP_OP_EXP + 1: st[sp - 1] = log(st[sp - 1]); pc++; break;
            case SP_OP_EXP + 2: st[sp - 1] = sqrt(st[sp - 1]); pc++; break;
            case SP_OP_EXP + 3: st[sp - 1] = sin(st[sp - 1]); pc++; break;
            case SP_OP_EXP + 4: st[sp - 1] = cos(st[sp - 1]); pc++; break;
            case SP_OP_EXP + 5: st[sp - 1] = tan(st[sp - 1]); pc++; break;
            case SP_OP_EXP + 6: st[sp - 1] = fabs(st[sp - 1]); pc++; break;
            case SP_OP_EXP + 7: st[sp - 1] = log10(st[sp - 1]); pc++; break;
            case SP_OP_EXP + 8: st[sp - 1] = floor(st[sp - 1]); pc++; break;
            case SP_OP_CEIL: st[sp - 1] = ceil(st[sp - 1]); pc++; break;
            default: {
                // binary operators
                const double b = st[sp - 1], a = st[sp - 2];
                double r;
                switch (op) {
                    case SP_OP_ADD: r = a + b; break;
                    case SP_OP_SUB: r = a - b; break;
                    case SP_OP_MUL: r = a * b; break;
                    case SP_OP_DIV: r = a / b; break;
                    case SP_OP_POW: r = pow(a, b); break;
                    case SP_OP_LT: r = a < b ? 1.0 : 0.0; break;
                    case SP_OP_LT + 1: r = a <= b ? 1.0 : 0.0; break;
                    case SP_OP_LT + 2: r = a > b ? 1.0 : 0.0; break;
                    case SP_OP_LT + 3: r = a >= b ? 1.0 : 0.0; break;
                    case SP_OP_LT + 4: r = a == b ? 1.0 : 0.0; break;
                    case SP_OP_NE: r = a != b ? 1.0 : 0.0; break;
                    case SP_OP_AND: r = (a != 0.0 && b != 0.0) ? 1.0 : 0.0; break;
                    default: r = (a != 0.0 || b != 0.0) ? 1.0 : 0.0; break;   // SP_OP_OR
                }
                st[sp - 2] = r;
                sp--;
                pc++;
                break;
            }
        }
    }
}

}  // namespace spg
