% advection/outputStep.m:53-66: nodal values evaluated on the device and written by the
% library's writer thread (dgadv_output); the call only enqueues, the time loop goes on.
function problemData = outputStep(problemData, nStep)
if problemData.isVisSol && mod(nStep, problemData.outputFrequency) == 0
  dgadv_mex('output', problemData.gpu, 'u_h', problemData.outputBasename, nStep, ...
            outputTypeBits(problemData.outputTypes));
end % if
end % function
