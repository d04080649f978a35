function problemData = outputStep(problemData, nStep)
if problemData.isVisSol && mod(nStep, problemData.outputFrequency) == 0
  problemData.cDisc = dgadv_mex('get_state', problemData.gpu, problemData.K, problemData.N);
  visualizeDataLagr(problemData.g, projectDataDisc2DataLagr(problemData.cDisc), 'u_h', ...
                    problemData.outputBasename, nStep, problemData.outputTypes);
end % if
end % function
