% advection/solveSubStep.m:57-99 (mass solve, time-derivative limiting, SSP update, solution
% limiting) for every stage of step nStep, enqueued at the first sub-step as one call: the
% stages are one chain of kernels on the device (one CUDA graph), so no stage state crosses the
% gateway.  The step's state stays on the device until get_state reads it.
function problemData = solveSubStep(problemData, nStep, nSubStep)
if nSubStep == 1
  dgadv_mex('step', problemData.gpu, 1, nStep - 1, problemData.tau);
end % if
end % function
