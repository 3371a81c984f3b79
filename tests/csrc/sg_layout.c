/* Prints the sizes and field offsets of the structs of sdem_surrogate.h, so
 * the ctypes mirrors can be checked against the compiler's layout. */
#include <stddef.h>
#include <stdio.h>

#include "../../include/sdem_surrogate.h"

#define F(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))

int main(void) {
    printf("sdem_sg_grid %zu\n", sizeof(sdem_sg_grid));
    F(sdem_sg_grid, cell); F(sdem_sg_grid, cutoff); F(sdem_sg_grid, scale); F(sdem_sg_grid, dim);
    printf("sdem_sg_operand %zu\n", sizeof(sdem_sg_operand));
    F(sdem_sg_operand, idx); F(sdem_sg_operand, ld); F(sdem_sg_operand, width); F(sdem_sg_operand, nseg);
    F(sdem_sg_operand, trans);
    printf("sdem_sg_box %zu\n", sizeof(sdem_sg_box));
    F(sdem_sg_box, hi);
    printf("sdem_sg_epilogue %zu\n", sizeof(sdem_sg_epilogue));
    F(sdem_sg_epilogue, relu); F(sdem_sg_epilogue, accumulate); F(sdem_sg_epilogue, mask);
    F(sdem_sg_epilogue, ld_mask); F(sdem_sg_epilogue, out); F(sdem_sg_epilogue, ld_out);
    F(sdem_sg_epilogue, out_bf); F(sdem_sg_epilogue, ld_out_bf); F(sdem_sg_epilogue, resid);
    F(sdem_sg_epilogue, ld_resid); F(sdem_sg_epilogue, res_out); F(sdem_sg_epilogue, ld_res_out);
    F(sdem_sg_epilogue, res_out_bf); F(sdem_sg_epilogue, ld_res_out_bf);
    return 0;
}
