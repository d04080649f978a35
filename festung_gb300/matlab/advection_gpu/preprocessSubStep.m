% advection/preprocessSubStep.m:56-99 assembles the stage operators (G, R, K_D, K_N, L).  On the
% device the operator is matrix-free inside the stage kernel, with the velocity factors uploaded
% once by preprocessProblem and the source / boundary terms by set_source_terms: nothing to do.
function problemData = preprocessSubStep(problemData, nStep, nSubStep) %#ok<INUSD>
end % function
