% Configuration of the advection_gpu problem: the advection problem's defaults and test cases
% (advection/configureProblem.m) on triangles, plus the device options.
function problemData = configureProblem(problemData)
problemData = setdefault(problemData, 'isQuadri', false);
assert(~problemData.isQuadri, 'advection_gpu runs on triangles only.')
problemData = setdefault(problemData, 'isVisSol', false);
problemData = setdefault(problemData, 'precision', 'fp64');   % 'fp64' | 'fp32'
problemData = setdefault(problemData, 'device', 0);
problemData = setdefault(problemData, 'gpuFlags', 0);
problemData = execin('advection/configureProblem', problemData);
end % function
