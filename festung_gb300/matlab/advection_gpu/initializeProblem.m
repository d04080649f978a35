% Initial data (advection/initializeProblem.m:46-86): L2 projection, upload, initial limiting.
function problemData = initializeProblem(problemData)
problemData.isFinished = false;
problemData.cDisc = projectFuncCont2DataDisc(problemData.g, problemData.c0Cont, problemData.qOrd, ...
                                             problemData.hatM, problemData.basesOnQuad);
dgadv_mex('set_state', problemData.gpu, problemData.cDisc);
if problemData.isSlopeLim
  dgadv_mex('limit_state', problemData.gpu, 0);
  problemData.cDisc = dgadv_mex('get_state', problemData.gpu, problemData.K, problemData.N);
end % if
if problemData.isVisSol   % advection/initializeProblem.m:80-86
  dgadv_mex('output', problemData.gpu, 'u_h', problemData.outputBasename, 0, ...
            outputTypeBits(problemData.outputTypes));
end % if
end % function
