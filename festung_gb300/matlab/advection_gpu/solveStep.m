% One SSP-RK step with all its stages on the device (advection/solveStep.m:57-73).
function problemData = solveStep(problemData, nStep)
dgadv_mex('step', problemData.gpu, 1, nStep - 1, problemData.tau);
end % function
