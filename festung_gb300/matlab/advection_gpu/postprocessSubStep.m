% advection/postprocessSubStep.m:55-57: the sub-step loop ends after the sub-step that ran the
% whole step on the device.
function problemData = postprocessSubStep(problemData, nStep, nSubStep) %#ok<INUSD>
problemData.isSubSteppingFinished = true;
end % function
