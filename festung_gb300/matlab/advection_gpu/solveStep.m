% One SSP-RK step (advection/solveStep.m:57-73): the RK tables and the sub-step loop of the
% reference.  The device runs every stage of the step as one chain of kernels, so the first
% sub-step enqueues the whole step (solveSubStep.m) and the loop ends there.
function problemData = solveStep(problemData, nStep)
[problemData.t, problemData.omega] = rungeKuttaExplicit(problemData.ordRK, problemData.tau, ...
                                                        (nStep - 1) * problemData.tau);
problemData.isSubSteppingFinished = false;
problemData = iterateSubSteps(problemData, nStep, problemData.subStepHandles);
end % function
