% Output, final state and L2 error (advection/postprocessProblem.m:43-82); releases the device
% handle once the output files are written.
function problemData = postprocessProblem(problemData)
if problemData.isVisSol
  dgadv_mex('output', problemData.gpu, 'u_h', problemData.outputBasename, problemData.numSteps, ...
            outputTypeBits(problemData.outputTypes));
  dgadv_mex('output_wait', problemData.gpu);
end % if
problemData.cDisc = dgadv_mex('get_state', problemData.gpu, problemData.K, problemData.N);
dgadv_mex('destroy', problemData.gpu);
if problemData.isAnalytical
  problemData.error = computeL2Error(problemData.g, problemData.cDisc, ...
    @(x1,x2) problemData.cCont(problemData.tEnd, x1, x2), problemData.qOrd, problemData.basesOnQuad);
else
  problemData.error = computeL2Error(problemData.g, problemData.cDisc, problemData.c0Cont, ...
    problemData.qOrd, problemData.basesOnQuad);
end % if
fprintf('L2 error: %g\n', problemData.error);
end % function
