"""lex_gb300: LEX's fully compressible dynamical-core step on GB300.

Modules (imported on demand; the native library is loaded by the first call that needs it):

    solver                 Solver: one context of liblexgb.so (state, base state, steps, budgets,
                           checkpoints, reverse mode, Smagorinsky constant)
    one_sprint_functions   drop-in for LEX's one_sprint_functions.py (ws_rk3_big_step,
                           ws_rk3_sprint, ws_rk3_sprint_dl, get_first_step_flux)
    write_netcdf, write_zarr   LEX's output writers (save2nc, save2nc_base, save2zarr)
    autograd               the big step as a torch.autograd operation (state and Cs)
    sgs_cnn                the learned SGS network on the library's BF16 tensor-core kernels
    learned_sgs            training data, training through the solver, evaluation
    gradcheck              gradient of a 600 s rollout against finite differences
    workload               warm-bubble initial states
    build                  builds liblexgb.so (nvcc, sm_103a)
"""
